// tx_alpha.cuh -- per-block device code for BC4 / BC5 (alpha::compress_bc3 on
// channel 0, and on channels 0 and 1; lib/src/lib.rs:199-204,
// lib/src/alpha.rs:187-256), shared by k_alpha and the batch kernel.
// Input is RGBA8 (the reference's layout, lib/src/lib.rs:323) or native
// R8 / RG8 rows (16 or 32 bytes per block instead of 64).
#pragma once
#include "tx_device.cuh"

namespace tx {

// Native single-/two-channel rows: 4 or 8 bytes per block row.
template <int CH>
__device__ __forceinline__ uint32_t load_block_native(const SrcDesc &s, size_t b, uint32_t (&r8)[4], uint32_t (&g8)[4]) {
    uint32_t bx, by;
    block_coords(s, b, bx, by);
    const uint32_t x0 = 4 * bx;
    uint32_t mask = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        r8[r] = 0; g8[r] = 0;
        const uint32_t y = 4 * by + r;
        if (y >= s.height) continue;
        const uint8_t *row = s.base + (size_t)y * s.pitch + (size_t)CH * x0;
        if (s.vec16 && x0 + 4 <= s.width) {
            if (CH == 1) {
                r8[r] = __ldcs(reinterpret_cast<const unsigned int *>(row));
            } else {
                const uint2 v = __ldcs(reinterpret_cast<const uint2 *>(row));
                r8[r] = __byte_perm(v.x, v.y, 0x6420);
                g8[r] = __byte_perm(v.x, v.y, 0x7531);
            }
            mask |= 0xFu << (4 * r);
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (x0 + c < s.width) {
                    r8[r] |= (uint32_t)row[CH * c] << (8 * c);
                    if (CH == 2) g8[r] |= (uint32_t)row[CH * c + 1] << (8 * c);
                    mask |= 1u << (4 * r + c);
                }
            }
        }
    }
    return mask;
}

// Encode and store block b.
template <int FMT, int CH>
__device__ __forceinline__ void alpha_block(const SrcDesc &src, size_t b, uint8_t *out) {
    uint32_t v0[4], v1[4], mask;
    if (CH == 4) {
        uint32_t px[16];
        mask = load_block_rgba(src, b, px);
        channel_words(px, 0, v0);
        if (FMT == BC5) channel_words(px, 1, v1);
    } else {
        mask = load_block_native<CH>(src, b, v0, v1);
    }
    const uint2 r = encode_bc3_alpha(v0, mask);
    if (FMT == BC4) {
        __stcs(reinterpret_cast<uint2 *>(out) + b, r);
    } else {
        const uint2 g = encode_bc3_alpha(v1, mask);
        __stcs(reinterpret_cast<uint4 *>(out) + b, make_uint4(r.x, r.y, g.x, g.y));
    }
}

}  // namespace tx
