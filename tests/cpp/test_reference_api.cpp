// The reference's own unit tests (lib/src/lib.rs:342-505) restated against the
// C++ mirror of its API (include/texpresso.hpp).  Known-answer data comes from
// tests/golden/kat.json through the generated header kat_data.h.
#include <cstdio>
#include <cstring>
#include <vector>

#include "texpresso.hpp"
#include "kat_data.h"

using namespace texpresso;

static int failures = 0;
#define EXPECT(cond)                                                        \
    do {                                                                    \
        if (!(cond)) {                                                      \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);     \
            ++failures;                                                     \
        }                                                                   \
    } while (0)

static void test_storage_requirements() {
    EXPECT(Format(Format::Bc1).compressed_size(16, 32) == 256);
    EXPECT(Format(Format::Bc1).compressed_size(15, 32) == 256);
    EXPECT(Format(Format::Bc2).compressed_size(16, 32) == 512);
    EXPECT(Format(Format::Bc2).compressed_size(15, 32) == 512);
    EXPECT(Format(Format::Bc3).compressed_size(16, 32) == 512);
    EXPECT(Format(Format::Bc3).compressed_size(15, 32) == 512);
    EXPECT(Format(Format::Bc4).compressed_size(16, 32) == 256);
    EXPECT(Format(Format::Bc4).compressed_size(15, 32) == 256);
    EXPECT(Format(Format::Bc5).compressed_size(16, 32) == 512);
    EXPECT(Format(Format::Bc5).compressed_size(15, 32) == 512);
}

static void execute_decompression_test(Format format, const KatSet &data) {
    std::vector<uint8_t> out(4 * 4 * 4);
    format.decompress(data.encoded, data.encoded_len, 4, 4, out.data(), out.size());
    EXPECT(std::memcmp(out.data(), data.decoded, 64) == 0);
}

static void execute_compression_test(Format format, const KatSet &data) {
    for (Algorithm algorithm : {Algorithm::ClusterFit, Algorithm::RangeFit, Algorithm::IterativeClusterFit}) {
        std::vector<uint8_t> out(format.block_size());
        Params p;
        p.algorithm = algorithm;
        p.weights = COLOUR_WEIGHTS_UNIFORM;
        p.weigh_colour_by_alpha = false;
        format.compress(data.decoded, 64, 4, 4, p, out.data(), out.size());
        EXPECT(out.size() == data.encoded_len && std::memcmp(out.data(), data.encoded, out.size()) == 0);
    }
}

static void test_bc1_decompression_height_not_multiple_of_4() {
    std::vector<uint8_t> out(4 * 4 * 6);
    Format(Format::Bc1).decompress(ODD_ENCODED, sizeof(ODD_ENCODED), 4, 6, out.data(), out.size());
    for (size_t i = 0; i < out.size(); i += 4) EXPECT(std::memcmp(out.data() + i, ODD_PIXEL, 4) == 0);
}

static void test_panics_become_exceptions() {
    std::vector<uint8_t> rgba(64), out(4);
    bool threw = false;
    try {
        Format(Format::Bc1).compress(rgba, 4, 4, Params{}, out);
    } catch (const Panic &e) {
        threw = e.status == TX_ERR_OUTPUT_TOO_SMALL;
    }
    EXPECT(threw);
}

int main() {
    test_storage_requirements();
    for (const KatSet &k : KAT_SETS) {
        Format f(static_cast<Format::Value>(k.format));
        execute_decompression_test(f, k);
        execute_compression_test(f, k);
    }
    test_bc1_decompression_height_not_multiple_of_4();
    test_panics_become_exceptions();
    std::printf("%s (%d failures)\n", failures ? "FAILED" : "OK", failures);
    return failures ? 1 : 0;
}
