// tx_decode.cu -- BCn decoders (Format::decompress, lib/src/lib.rs:124-156;
// decompress_block, lib/src/lib.rs:240-277; colourblock::decompress,
// lib/src/colourblock.rs:97-169; alpha::decompress_bc2/bc3,
// lib/src/alpha.rs:53-68, :258-304).  One thread per block; integer only.
#include "tx_device.cuh"
#include "tx_internal.h"

namespace tx {

__device__ __forceinline__ uint32_t expand565(uint32_t v) {
    const uint32_t r = (v >> 11) & 0x1Fu, g = (v >> 5) & 0x3Fu, b = v & 0x1Fu;
    return ((r << 3) | (r >> 2)) | (((g << 2) | (g >> 4)) << 8) | (((b << 3) | (b >> 2)) << 16) | 0xFF000000u;
}

// 16 RGBA8 pixels of a BC1/BC2/BC3 colour block.
__device__ __forceinline__ void decode_colour(uint2 blk, bool is_bc1, uint32_t (&px)[16]) {
    const uint32_t a = blk.x & 0xFFFFu, b = blk.x >> 16;
    uint32_t code[4];
    code[0] = expand565(a);
    code[1] = expand565(b);
    uint32_t c2 = 0, c3 = 0;
    const bool three = is_bc1 && a <= b;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const uint32_t c = (code[0] >> (8 * ch)) & 0xFFu, d = (code[1] >> (8 * ch)) & 0xFFu;
        if (three) { c2 |= ((c + d) / 2) << (8 * ch); }
        else { c2 |= ((2 * c + d) / 3) << (8 * ch); c3 |= ((c + 2 * d) / 3) << (8 * ch); }
    }
    c2 |= 0xFF000000u;
    if (!three) c3 |= 0xFF000000u;
    code[2] = c2;
    code[3] = c3;
#pragma unroll
    for (int i = 0; i < 16; ++i) px[i] = code[(blk.y >> (2 * i)) & 3u];
}

__device__ __forceinline__ void decode_alpha8(uint2 blk, int ch, uint32_t (&px)[16]) {
    const int a0 = (int)(blk.x & 0xFFu), a1 = (int)((blk.x >> 8) & 0xFFu);
    int code[8];
    code[0] = a0; code[1] = a1;
    if (a0 <= a1) {
#pragma unroll
        for (int i = 1; i < 5; ++i) code[1 + i] = ((5 - i) * a0 + i * a1) / 5;
        code[6] = 0; code[7] = 255;
    } else {
#pragma unroll
        for (int i = 1; i < 7; ++i) code[1 + i] = ((7 - i) * a0 + i * a1) / 7;
    }
    const uint64_t bits = ((uint64_t)blk.x >> 16) | ((uint64_t)blk.y << 16);
    const uint32_t sh = 8u * (uint32_t)ch, keep = ~(0xFFu << sh);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const uint32_t v = (uint32_t)code[(bits >> (3 * i)) & 7u];
        px[i] = (px[i] & keep) | (v << sh);
    }
}

template <int FMT>
__global__ void __launch_bounds__(128) k_decode(const uint8_t *__restrict__ data, size_t blocks_wide,
                                                size_t block_rows, size_t width, size_t height,
                                                uint8_t *__restrict__ out, size_t out_pitch, size_t out_len) {
    const size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= blocks_wide * block_rows) return;
    const size_t bx = b % blocks_wide, by = b / blocks_wide;
    uint32_t px[16];
    if (FMT == BC1 || FMT == BC2 || FMT == BC3) {
        const uint2 c = reinterpret_cast<const uint2 *>(data + b * block_bytes(FMT))[FMT == BC1 ? 0 : 1];
        decode_colour(c, FMT == BC1, px);
    } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) px[i] = 0xFF000000u;
    }
    const uint2 a = reinterpret_cast<const uint2 *>(data + b * block_bytes(FMT))[0];
    if (FMT == BC2) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const uint32_t q = ((i < 8 ? a.x : a.y) >> (4 * (i & 7))) & 0xFu;
            px[i] = (px[i] & 0x00FFFFFFu) | ((q | (q << 4)) << 24);
        }
    } else if (FMT == BC3) {
        decode_alpha8(a, 3, px);
    } else if (FMT == BC4) {
        decode_alpha8(a, 0, px);
#pragma unroll
        for (int i = 0; i < 16; ++i) { const uint32_t r = px[i] & 0xFFu; px[i] = 0xFF000000u | r | (r << 8) | (r << 16); }
    } else if (FMT == BC5) {
        decode_alpha8(a, 0, px);
        decode_alpha8(reinterpret_cast<const uint2 *>(data + b * 16)[1], 1, px);
    }
#pragma unroll
    for (int py = 0; py < 4; ++py) {
        const size_t y = 4 * by + py;
        if (y >= height) continue;
#pragma unroll
        for (int pxi = 0; pxi < 4; ++pxi) {
            const size_t x = 4 * bx + pxi;
            const size_t o = y * out_pitch + 4 * x;
            if (x < width && o + 4 <= out_len) {
                uint8_t *d = out + o;
                const uint32_t v = px[4 * py + pxi];
                d[0] = (uint8_t)v; d[1] = (uint8_t)(v >> 8); d[2] = (uint8_t)(v >> 16); d[3] = (uint8_t)(v >> 24);
            }
        }
    }
}

cudaError_t launch_decode(int fmt, const uint8_t *data, size_t blocks_wide, size_t block_rows, size_t width,
                          size_t height, uint8_t *out, size_t out_pitch, size_t out_len, cudaStream_t st) {
    const size_t n = blocks_wide * block_rows;
    if (n == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n + 127) / 128);
    switch (fmt) {
    case BC1: k_decode<BC1><<<grid, 128, 0, st>>>(data, blocks_wide, block_rows, width, height, out, out_pitch, out_len); break;
    case BC2: k_decode<BC2><<<grid, 128, 0, st>>>(data, blocks_wide, block_rows, width, height, out, out_pitch, out_len); break;
    case BC3: k_decode<BC3><<<grid, 128, 0, st>>>(data, blocks_wide, block_rows, width, height, out, out_pitch, out_len); break;
    case BC4: k_decode<BC4><<<grid, 128, 0, st>>>(data, blocks_wide, block_rows, width, height, out, out_pitch, out_len); break;
    case BC5: k_decode<BC5><<<grid, 128, 0, st>>>(data, blocks_wide, block_rows, width, height, out, out_pitch, out_len); break;
    default: return cudaErrorInvalidValue;
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace tx
