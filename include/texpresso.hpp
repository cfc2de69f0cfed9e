// texpresso.hpp -- C++ mirror of texpresso's public API (lib/src/lib.rs) over
// the C ABI of libtexpresso_gb300.so.
//
// Same names and argument meaning as the Rust crate:
//   texpresso::Format::{Bc1..Bc5} with compress, compress_block_masked,
//   decompress, decompress_block, block_size, compressed_size;
//   texpresso::Params, texpresso::Algorithm, COLOUR_WEIGHTS_UNIFORM,
//   COLOUR_WEIGHTS_PERCEPTUAL, num_blocks.
// Where the reference panics (lib/src/lib.rs:295, slice bounds) these throw
// texpresso::Panic carrying the C status code.  Header-only; link with
// -ltexpresso_gb300.
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "texpresso_gb300.h"

namespace texpresso {

struct Panic : std::runtime_error {
    int status;
    Panic(int s, const char *what)
        : std::runtime_error(std::string(what) + ": " + tx_status_string(s)), status(s) {}
};

inline void check(int rc, const char *what) {
    if (rc != TX_OK) throw Panic(rc, what);
}

// lib/src/lib.rs:49-65
enum class Algorithm : int32_t {
    RangeFit = TX_RANGE_FIT,
    ClusterFit = TX_CLUSTER_FIT,
    IterativeClusterFit = TX_ITERATIVE_CLUSTER_FIT,
};

// lib/src/lib.rs:68-74
using ColourWeights = std::array<float, 3>;
inline constexpr ColourWeights COLOUR_WEIGHTS_UNIFORM = {1.0f, 1.0f, 1.0f};
inline constexpr ColourWeights COLOUR_WEIGHTS_PERCEPTUAL = {0.2126f, 0.7152f, 0.0722f};

// lib/src/lib.rs:76-100
struct Params {
    Algorithm algorithm = Algorithm::ClusterFit;
    ColourWeights weights = COLOUR_WEIGHTS_PERCEPTUAL;
    bool weigh_colour_by_alpha = false;

    tx_params c() const {
        tx_params p;
        p.algorithm = static_cast<int32_t>(algorithm);
        for (int i = 0; i < 3; ++i) p.weights[i] = weights[i];
        p.weigh_colour_by_alpha = weigh_colour_by_alpha ? 1 : 0;
        return p;
    }
};

// lib/src/lib.rs:103-105
inline size_t num_blocks(size_t size) { return tx_num_blocks(size); }

// lib/src/lib.rs:39-46 and impl Format (:117-336)
class Format {
  public:
    enum Value : int { Bc1 = TX_FORMAT_BC1, Bc2 = TX_FORMAT_BC2, Bc3 = TX_FORMAT_BC3, Bc4 = TX_FORMAT_BC4, Bc5 = TX_FORMAT_BC5 };
    constexpr Format(Value v) : v_(v) {}
    constexpr operator Value() const { return v_; }

    size_t block_size() const { return tx_block_size(v_); }
    size_t compressed_size(size_t width, size_t height) const { return tx_compressed_size(v_, width, height); }

    // Format::compress (lib/src/lib.rs:287-335)
    void compress(const uint8_t *rgba, size_t rgba_len, size_t width, size_t height, const Params &params,
                  uint8_t *output, size_t output_len) const {
        const tx_params p = params.c();
        check(tx_compress(v_, rgba, rgba_len, width, height, &p, output, output_len), "Format::compress");
    }
    template <class In, class Out>
    void compress(const In &rgba, size_t width, size_t height, const Params &params, Out &output) const {
        compress(rgba.data(), rgba.size(), width, height, params, output.data(), output.size());
    }

    // Format::compress_block_masked (lib/src/lib.rs:188-234)
    void compress_block_masked(const std::array<uint8_t, 64> &rgba, uint32_t mask, const Params &params,
                               uint8_t *output, size_t output_len) const {
        const tx_params p = params.c();
        check(tx_compress_block_masked(v_, rgba.data(), mask, &p, output, output_len),
              "Format::compress_block_masked");
    }

    // Format::decompress (lib/src/lib.rs:124-156)
    void decompress(const uint8_t *data, size_t data_len, size_t width, size_t height, uint8_t *output,
                    size_t output_len) const {
        check(tx_decompress(v_, data, data_len, width, height, output, output_len), "Format::decompress");
    }
    template <class In, class Out>
    void decompress(const In &data, size_t width, size_t height, Out &output) const {
        decompress(data.data(), data.size(), width, height, output.data(), output.size());
    }

    // Format::decompress_block (lib/src/lib.rs:240-277)
    std::array<uint8_t, 64> decompress_block(const uint8_t *block, size_t block_len) const {
        std::array<uint8_t, 64> out{};
        check(tx_decompress_block(v_, block, block_len, out.data()), "Format::decompress_block");
        return out;
    }

  private:
    Value v_;
};

}  // namespace texpresso
