// Block coordinates by the precomputed reciprocal of the row width
// (set_blocks_wide / block_coords in tx_device.cuh), run on the host against
// plain division: every row width up to 2^16 and a spread of larger ones,
// block numbers at and around every multiple of the width near 0, near 2^32
// and at random.
#include "tx_device.cuh"

#include <cstdio>
#include <random>

int main() {
    std::mt19937_64 rng(3);
    long checked = 0, bad = 0;
    auto check = [&](const tx::SrcDesc &s, uint64_t n) {
        uint32_t bx, by;
        tx::block_coords(s, (size_t)n, bx, by);
        ++checked;
        if (by != (uint32_t)(n / s.blocks_wide) || bx != (uint32_t)(n % s.blocks_wide)) {
            if (++bad < 8) printf("width %u block %llu: (%u, %u)\n", s.blocks_wide, (unsigned long long)n, bx, by);
        }
    };
    for (uint64_t w = 1; w <= (1u << 20); w = w < 65536 ? w + 1 : w + 1 + (rng() % 4096)) {
        tx::SrcDesc s{};
        tx::set_blocks_wide(s, (uint32_t)w);
        for (uint64_t k = 0; k < 4; ++k)
            for (int d = -1; d <= 1; ++d) {
                const int64_t n = (int64_t)(k * w) + d;
                if (n >= 0) check(s, (uint64_t)n);
            }
        const uint64_t top = 0xFFFFFFFFull;
        for (uint64_t q = top / w - 1; q <= top / w + 1; ++q)
            for (int d = -1; d <= 1; ++d) {
                const int64_t n = (int64_t)(q * w) + d;
                if (n >= 0 && (uint64_t)n <= top) check(s, (uint64_t)n);
            }
        check(s, top);
        for (int r = 0; r < 16; ++r) check(s, rng() & top);
        check(s, top + 1 + (rng() % 1000000));  // beyond 32 bits: the 64-bit path
    }
    printf("checked %ld block numbers, %ld wrong\n", checked, bad);
    return bad ? 1 : 0;
}
