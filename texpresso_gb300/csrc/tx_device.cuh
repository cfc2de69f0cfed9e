// tx_device.cuh -- device-side building blocks shared by the BCn kernels.
//
// Every translation unit that includes this file is compiled with
// -fmad=false -prec-div=true -prec-sqrt=true -ftz=false: a*b+c is never fused,
// division and square root are IEEE round-to-nearest, subnormals are kept.
// That reproduces the reference's scalar f32 arithmetic (Rust never contracts;
// lib/src/math/vec3.rs, lib/src/math/vec4.rs) bit for bit.
#pragma once

#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

namespace tx {

enum Format : int { BC1 = 0, BC2 = 1, BC3 = 2, BC4 = 3, BC5 = 4 };
enum Algorithm : int { RANGE_FIT = 0, CLUSTER_FIT = 1, ITERATIVE_CLUSTER_FIT = 2 };

// Kernel-side copy of the caller's Params (lib/src/lib.rs:76-90).
struct DevParams {
    float w[3];
    int alpha_weighted;
};

// Where a kernel reads its pixels from.
struct SrcDesc {
    const uint8_t *base;   // image (mode 0) or packed 64-byte blocks (mode 1)
    const uint32_t *masks; // mode 1: per-block valid masks (nullptr = all valid)
    size_t pitch;          // mode 0: bytes between rows
    uint32_t width, height;
    uint32_t blocks_wide;  // num_blocks(width)
    uint32_t bw_magic, bw_shift, bw_flags;  // division by blocks_wide (set_blocks_wide)
    int channels;          // 4 = RGBA8, 1 = R8, 2 = RG8
    int vec16;             // mode 0, RGBA8: rows 16-byte aligned -> 128-bit loads
    int mode;              // 0 image, 1 block list
};

// blocks_wide and the multiplier that divides 32-bit block numbers by it:
// q = umulhi(n, magic) >> shift, or with the add step (flags bit 0)
// q = (((n - t) >> 1) + t) >> shift, t = umulhi(n, magic), or n >> shift for a
// power of two (flags bit 1) -- division by an invariant integer with a
// rounded-up reciprocal (Granlund and Montgomery), exact for every 32-bit n.
inline void set_blocks_wide(SrcDesc &s, uint32_t bw) {
    s.blocks_wide = bw;
    s.bw_magic = 0;
    s.bw_shift = 0;
    s.bw_flags = 2;
    if (bw == 0) return;
    const uint32_t l = 31u - (uint32_t)__builtin_clz(bw);
    s.bw_shift = l;
    if ((bw & (bw - 1)) == 0) return;
    const uint64_t num = (uint64_t)1 << (32 + l);
    uint64_t m = num / bw;
    const uint64_t rem = num - m * bw;
    if (bw - rem < ((uint64_t)1 << l)) {
        s.bw_flags = 0;
    } else {
        m = 2 * m + (2 * rem >= bw ? 1u : 0u);
        s.bw_flags = 1;
    }
    s.bw_magic = (uint32_t)(m + 1);
}

// Block column and row of block b.
__host__ __device__ __forceinline__ uint32_t umulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ void block_coords(const SrcDesc &s, size_t b, uint32_t &bx, uint32_t &by) {
    if (b <= 0xFFFFFFFFull) {
        const uint32_t n = (uint32_t)b;
        uint32_t q;
        if (s.bw_flags & 2u) {
            q = n >> s.bw_shift;
        } else {
            const uint32_t t = umulhi32(n, s.bw_magic);
            q = (s.bw_flags & 1u) ? ((((n - t) >> 1) + t) >> s.bw_shift) : (t >> s.bw_shift);
        }
        by = q;
        bx = n - q * s.blocks_wide;
    } else {
        by = (uint32_t)(b / s.blocks_wide);
        bx = (uint32_t)(b % s.blocks_wide);
    }
}

__host__ __device__ constexpr int block_bytes(int fmt) { return (fmt == BC1 || fmt == BC4) ? 8 : 16; }

// ---------------------------------------------------------------------------
// exact scalar helpers (lib/src/math.rs:100-102, lib/src/math/vec4.rs:94-110)

__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }   // == 1.0f / x

// Paired f32 operations (sm_100+): each lane is the IEEE round-to-nearest
// operation of the scalar form.  A paired multiply whose result feeds a
// paired add can still end up fused into one multiply-add (measured: the
// rounding of a squared-distance sum changed), so use them only where no
// multiply feeds an add.
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_rn(float x) { return __fsqrt_rn(x); }

// f32_to_i32_clamped: roundf(a).max(0).min(limit) as i32 (max/min drop NaN).
__device__ __forceinline__ int f32_to_i32_clamped(float a, int limit) {
    return (int)fminf(fmaxf(roundf(a), 0.0f), (float)limit);
}

// u8 -> [0,1] exactly as colourset.rs:65-67 (f32::from(v) / 255f32).
__device__ __forceinline__ float unorm8(uint32_t v) { return div_rn((float)v, 255.0f); }

// ---------------------------------------------------------------------------
// packing (lib/src/colourblock.rs:28-94)

__device__ __forceinline__ uint32_t pack_565(float x, float y, float z) {
    uint32_t r = (uint32_t)f32_to_i32_clamped(31.0f * x, 31);
    uint32_t g = (uint32_t)f32_to_i32_clamped(63.0f * y, 63);
    uint32_t b = (uint32_t)f32_to_i32_clamped(31.0f * z, 31);
    return (r << 11) | (g << 5) | b;
}

// Swap 2-bit indices 0 <-> 1 (write3's remap), 16 packed indices at once.
__device__ __forceinline__ uint32_t swap01_2bit(uint32_t w) {
    // an index is 0 or 1 when its high bit is clear; flipping its low bit swaps it
    uint32_t hi = (w >> 1) & 0x55555555u;
    return w ^ (~hi & 0x55555555u);
}

// write3: endpoints a,b (565) and 16 2-bit indices (pixel i at bits 2i).
__device__ __forceinline__ uint2 write3(uint32_t a, uint32_t b, uint32_t idx) {
    if (a > b) { uint32_t t = a; a = b; b = t; idx = swap01_2bit(idx); }
    return make_uint2(a | (b << 16), idx);
}

// write4: a<b swaps and flips bit 0 of every index; a==b zeroes the indices.
__device__ __forceinline__ uint2 write4(uint32_t a, uint32_t b, uint32_t idx) {
    if (a < b) { uint32_t t = a; a = b; b = t; idx ^= 0x55555555u; }
    else if (a == b) { idx = 0; }
    return make_uint2(a | (b << 16), idx);
}

// ---------------------------------------------------------------------------
// block gather (lib/src/lib.rs:305-333): 16 RGBA8 pixels + valid mask.

__device__ __forceinline__ uint32_t ld_u32_any(const uint8_t *p) {
    // p is 4-byte aligned when the image base is; fall back to bytes otherwise
    if ((reinterpret_cast<uintptr_t>(p) & 3u) == 0) return __ldg(reinterpret_cast<const uint32_t *>(p));
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// Load the 16 pixels of block `b` into px[] (pixel 4*y+x), return the mask.
// Masked pixels read as 0; the reference never looks at them.
__device__ __forceinline__ uint32_t load_block_rgba(const SrcDesc &s, size_t b, uint32_t (&px)[16]) {
    if (s.mode == 1) {
        const uint4 *q = reinterpret_cast<const uint4 *>(s.base + 64 * b);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            uint4 v = __ldg(q + r);
            px[4 * r + 0] = v.x; px[4 * r + 1] = v.y; px[4 * r + 2] = v.z; px[4 * r + 3] = v.w;
        }
        return s.masks ? (__ldg(s.masks + b) & 0xFFFFu) : 0xFFFFu;
    }
    uint32_t bx, by;
    block_coords(s, b, bx, by);
    const uint32_t x0 = 4 * bx;
    uint32_t mask = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const uint32_t y = 4 * by + r;
        if (y < s.height) {
            const uint8_t *row = s.base + (size_t)y * s.pitch + 4 * (size_t)x0;
            if (s.vec16 && x0 + 4 <= s.width) {
                uint4 v = __ldcs(reinterpret_cast<const uint4 *>(row));
                px[4 * r + 0] = v.x; px[4 * r + 1] = v.y; px[4 * r + 2] = v.z; px[4 * r + 3] = v.w;
                mask |= 0xFu << (4 * r);
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if (x0 + c < s.width) { px[4 * r + c] = ld_u32_any(row + 4 * c); mask |= 1u << (4 * r + c); }
                    else px[4 * r + c] = 0;
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < 4; ++c) px[4 * r + c] = 0;
        }
    }
    return mask;
}

// Expand a 4-bit pixel mask into byte lanes (0xFF per valid pixel).
__device__ __forceinline__ uint32_t nibble_to_bytemask(uint32_t nib) {
    return ((nib * 0x00204081u) & 0x01010101u) * 0xFFu;
}

// ---------------------------------------------------------------------------
// BC2 alpha (lib/src/alpha.rs:27-51)

__device__ __forceinline__ uint32_t bc2_quant(uint32_t a) {
    return (uint32_t)f32_to_i32_clamped((float)a * (15.0f / 255.0f), 15);
}

__device__ __forceinline__ uint2 encode_bc2_alpha(const uint32_t (&px)[16], uint32_t mask) {
    uint32_t lo = 0, hi = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        uint32_t q = ((mask >> i) & 1u) ? bc2_quant(px[i] >> 24) : 0u;
        if (i < 8) lo |= q << (4 * i); else hi |= q << (4 * (i - 8));
    }
    return make_uint2(lo, hi);
}

// ---------------------------------------------------------------------------
// BC3/BC4/BC5 alpha block (lib/src/alpha.rs:70-256): codebook search on
// sorted thresholds, four pixels per 32-bit word (byte c of v[r] = pixel 4r+c).
//
// fit_codes (alpha.rs:79-117) gives each pixel the first code of least
// squared distance.  With the 8 codes sorted by (value, index), a code whose
// value equals its predecessor's can never be chosen (the predecessor has the
// same distance and a smaller index), so it takes the predecessor's place.
// Between sorted neighbours a <= b a pixel x prefers b iff 2x > a + b, or
// 2x == a + b and b's index is smaller, i.e. iff x >= T = (a + b + 2 - [ib < ia]) / 2
// (integer division).  T never decreases along the sorted list, and the
// distances are unimodal in it, so the chosen code is the one at position
// #{j : x >= T_j}, found by a three-step binary search with per-byte
// compares.  T = 256 only arises between two 255s, which after the merge are
// the same code, so clamping T to 255 changes nothing.  Squared errors are
// x^2 - 2xv + v^2 summed with dp4a; the x^2 part is common to both
// codebooks.

// prmt.b32 in its generic mode: 4-bit selectors, bit 3 replicates the
// selected byte's sign bit.  (The host form lets the codebook builders below
// be checked on the CPU.)
__host__ __device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
#ifdef __CUDA_ARCH__
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
#else
    const uint64_t src = (uint64_t)a | ((uint64_t)b << 32);
    uint32_t d = 0;
    for (int k = 0; k < 4; ++k) {
        const uint32_t s = (sel >> (4 * k)) & 0xFu;
        uint32_t byte = (uint32_t)(src >> (8 * (s & 7u))) & 0xFFu;
        if (s & 8u) byte = (byte & 0x80u) ? 0xFFu : 0x00u;
        d |= byte << (8 * k);
    }
    return d;
#endif
}

__host__ __device__ __forceinline__ int popc32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

// Lane-wise minimum / maximum of two pairs of unsigned 16-bit values.
__device__ __forceinline__ uint32_t min_u16x2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ uint32_t max_u16x2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}

// 0xFF in every byte where x >= t (unsigned), else 0x00.
__host__ __device__ __forceinline__ uint32_t bytes_ge(uint32_t x, uint32_t t) {
    const uint32_t H = 0x80808080u;
    const uint32_t g = (x | H) - (t & ~H);         // top bit: low 7 bits of x >= those of t
    const uint32_t m = (x & ~t) | (~(x ^ t) & g);  // top bit: x >= t
    return prmt(m, 0u, 0xBA98u);                   // replicate each byte's top bit
}

struct AlphaBook {
    uint32_t t[7];             // thresholds, replicated in every byte
    uint32_t idx_lo, idx_hi;   // code index at sorted positions 0-3 / 4-7
    uint32_t val_lo, val_hi;   // code value at sorted positions 0-3 / 4-7
};

// 0xFF in every byte where x == y, else 0x00.
__host__ __device__ __forceinline__ uint32_t bytes_eq(uint32_t x, uint32_t y) {
    const uint32_t H = 0x80808080u, d = x ^ y;
    return prmt(~(((d | H) - 0x01010101u) | d) & H, 0u, 0xBA98u);
}

// The 7-value book (alpha.rs:237-242) without a sort: codes 2-7, the
// interpolants of min7..max7, rise strictly (max7 - min7 >= 7), and min5 <
// max5 (indices 0 and 1) go in front of the interpolants of equal value, so
// in (value, index) order min5 sits after the p0 interpolants below it and
// max5 after the p1 - 1 below it and min5.  One nibble selector per sorted
// position then gathers values and indices with prmt from the bytes
// [c2 c3 c4 c5 | c6 c7 min5 max5].  An interpolant equal to min5 or max5
// directly follows it and takes its index (the merge of make_book; values
// are distinct otherwise, so merges never chain).  Thresholds between
// neighbours (a, b) are (a + b + 2 - [ib < ia]) / 2 capped at 255: the
// rounded-up byte average, plus one when a + b is even and ib > ia.
__host__ __device__ __forceinline__ AlphaBook make_book7(uint32_t min5, uint32_t max5, const uint32_t (&c)[8]) {
    const uint32_t A = c[2] | c[3] << 8 | c[4] << 16 | c[5] << 24;
    const uint32_t B6 = c[6] | c[7] << 8 | 0xFFFF0000u;  // padding bytes never count as below
    const uint32_t n5 = min5 * 0x01010101u, x5 = max5 * 0x01010101u;
    const uint32_t p0 = (uint32_t)(popc32(~bytes_ge(A, n5)) + popc32(~bytes_ge(B6, n5))) >> 3;
    const uint32_t p1 = ((uint32_t)(popc32(~bytes_ge(A, x5)) + popc32(~bytes_ge(B6, x5))) >> 3) + 1u;
    uint32_t sel = 0x76543210u - (0x11111111u << (4 * p0 + 4)) - (p1 < 7u ? 0x11111111u << (4 * p1 + 4) : 0u);
    sel = (sel & ~(0xFu << (4 * p0))) | (6u << (4 * p0));
    sel = (sel & ~(0xFu << (4 * p1))) | (7u << (4 * p1));
    const uint32_t B = (B6 & 0xFFFFu) | min5 << 16 | max5 << 24;
    AlphaBook bk;
    bk.val_lo = prmt(A, B, sel & 0xFFFFu);
    bk.val_hi = prmt(A, B, sel >> 16);
    const uint32_t ilo = prmt(0x05040302u, 0x01000706u, sel & 0xFFFFu);
    const uint32_t ihi = prmt(0x05040302u, 0x01000706u, sel >> 16);
    // merge: equal to the predecessor's value -> the predecessor's index
    const uint32_t eq_lo = bytes_eq(bk.val_lo, prmt(bk.val_lo, ~bk.val_lo, 0x2104u));
    const uint32_t eq_hi = bytes_eq(bk.val_hi, prmt(bk.val_lo, bk.val_hi, 0x6543u));
    bk.idx_lo = (ilo & ~eq_lo) | (prmt(ilo, 0u, 0x2104u) & eq_lo);
    bk.idx_hi = (ihi & ~eq_hi) | (prmt(ilo, ihi, 0x6543u) & eq_hi);
    // thresholds of the pairs (s, s+1), s = 0-3 in the low word, 4-6 in the high
    const uint32_t rv_lo = prmt(bk.val_lo, bk.val_hi, 0x4321u), rv_hi = bk.val_hi >> 8;
    const uint32_t rx_lo = prmt(bk.idx_lo, bk.idx_hi, 0x4321u), rx_hi = bk.idx_hi >> 8;
    uint32_t T[2];
#pragma unroll
    for (int w = 0; w < 2; ++w) {
        const uint32_t a = w ? bk.val_hi : bk.val_lo, b = w ? rv_hi : rv_lo;
        const uint32_t xa = w ? bk.idx_hi : bk.idx_lo, xb = w ? rx_hi : rx_lo;
        const uint32_t up = (a | b) - (((a ^ b) >> 1) & 0x7F7F7F7Fu);   // (a + b + 1) >> 1
        const uint32_t ge = ~(((xb | 0x08080808u) - xa) >> 3) ^ 0xFFFFFFFFu;  // bit 0: ib >= ia
        // + 1 where a + b is even and ib > ia (ib == ia only for merged equal
        // values, where a + b is even too and the rule adds one as well)
        uint32_t inc = ~(a ^ b) & ge & 0x01010101u;
        inc &= ~bytes_eq(up, 0xFFFFFFFFu);  // 255 + 1 is capped at 255
        T[w] = up + inc;
    }
#pragma unroll
    for (int s = 0; s < 7; ++s) bk.t[s] = prmt(T[s >> 2], 0u, (uint32_t)(s & 3) * 0x1111u);
    return bk;
}

// The 5-value book (alpha.rs:227-234) needs no sort: its values run
// 0 (index 6), min5 (0), the four interpolants (2-5), max5 (1), 255 (7), with
// the interpolants strictly between min5 and max5 after fix_range.  The
// thresholds follow from the rule above with the index comparisons known; a
// min5 of 0 gets threshold 0 (index 0 always beats index 6), and a max5 of 255
// makes the last position index 1 again (the merge of equal values).
__host__ __device__ __forceinline__ AlphaBook make_book5(uint32_t min5, uint32_t max5, const uint32_t (&c)[8]) {
    AlphaBook bk;
    const uint32_t t[7] = {(min5 + 1u) >> 1,          (min5 + c[2] + 2u) >> 1, (c[2] + c[3] + 2u) >> 1,
                           (c[3] + c[4] + 2u) >> 1,   (c[4] + c[5] + 2u) >> 1, (c[5] + max5 + 1u) >> 1,
                           min((max5 + 257u) >> 1, 255u)};
#pragma unroll
    for (int j = 0; j < 7; ++j) bk.t[j] = t[j] * 0x01010101u;
    bk.idx_lo = 6u | (0u << 8) | (2u << 16) | (3u << 24);
    bk.idx_hi = 4u | (5u << 8) | (1u << 16) | ((max5 == 255u ? 1u : 7u) << 24);
    bk.val_lo = (min5 << 8) | (c[2] << 16) | (c[3] << 24);
    bk.val_hi = c[4] | (c[5] << 8) | (max5 << 16) | (255u << 24);
    return bk;
}

// Code index of every pixel (masked pixels: 0) and the book's share of the
// error, sum over valid pixels of v^2 - 2 x v (the x^2 part is left out).
__device__ __forceinline__ int fit_book(const uint32_t (&x)[4], const uint32_t (&vm)[4], const AlphaBook &bk,
                                        uint32_t (&idx)[4]) {
    uint32_t sv = 0, sxv = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const uint32_t m2 = bytes_ge(x[r], bk.t[3]);
        const uint32_t m1 = bytes_ge(x[r], (m2 & bk.t[5]) | (~m2 & bk.t[1]));
        const uint32_t hi = (m1 & bk.t[6]) | (~m1 & bk.t[4]);
        const uint32_t lo = (m1 & bk.t[2]) | (~m1 & bk.t[0]);
        const uint32_t m0 = bytes_ge(x[r], (m2 & hi) | (~m2 & lo));
        const uint32_t p = (m2 & 0x04040404u) | (m1 & 0x02020202u) | (m0 & 0x01010101u);
        const uint32_t q = (p | (p >> 4)) & 0x00FF00FFu;
        const uint32_t sel = (q | (q >> 8)) & 0xFFFFu;
        idx[r] = prmt(bk.idx_lo, bk.idx_hi, sel) & vm[r];
        const uint32_t v = prmt(bk.val_lo, bk.val_hi, sel) & vm[r];
        sv = __dp4a(v, v, sv);
        sxv = __dp4a(x[r] & vm[r], v, sxv);
    }
    return (int)sv - 2 * (int)sxv;
}

// fix_range (alpha.rs:70-77); min <= max on entry.
__host__ __device__ __forceinline__ void fix_range(int &mn, int &mx, int steps) {
    if (mx - mn < steps) mx = min(mn + steps, 255);
    if (mx - mn < steps) mn = max(mx - steps, 0);
}

// 3-bit indices of four pixels (one per byte) -> 12 bits.
__device__ __forceinline__ uint32_t pack3x4(uint32_t w) {
    return (w & 0x7u) | ((w >> 5) & 0x38u) | ((w >> 10) & 0x1C0u) | ((w >> 15) & 0xE00u);
}

__device__ __forceinline__ uint2 write_alpha_block(uint32_t a0, uint32_t a1, const uint32_t (&idx)[4]) {
    const uint32_t lo = pack3x4(idx[0]) | (pack3x4(idx[1]) << 12);  // pixels 0..7
    const uint32_t hi = pack3x4(idx[2]) | (pack3x4(idx[3]) << 12);  // pixels 8..15
    return make_uint2(a0 | (a1 << 8) | ((lo & 0xFFFFu) << 16), (lo >> 16) | (hi << 8));
}

// compress_bc3 for one channel: v = 16 packed values, mask = valid pixels.
// FULL: every pixel is valid (mask == 0xFFFF), so the byte masks fold away.
template <bool FULL>
__device__ __forceinline__ uint2 encode_bc3_alpha_t(const uint32_t (&v)[4], uint32_t mask) {
    uint32_t vm[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) vm[r] = FULL ? 0xFFFFFFFFu : nibble_to_bytemask((mask >> (4 * r)) & 0xFu);
    // Ranges (alpha.rs:194-212).  Masked pixels enter as 255 for the minima and
    // 0 for the maxima (the initial values).  min5 skips zeros: the minimum of
    // (x - 1) mod 256 plus one, where a zero becomes 255 and a masked pixel
    // 254 (= 255, the initial value); max5 skips 255s the same way with
    // (x + 1) mod 256.  Bytes are compared as even and odd 16-bit pairs.
    const uint32_t H = 0x80808080u;
    uint32_t mn7 = 0xFFFFFFFFu, mx7 = 0, mn5 = 0xFFFFFFFFu, mx5 = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const uint32_t lo7 = v[r] | ~vm[r], hi7 = v[r] & vm[r];
        const uint32_t lo5 = ((lo7 | H) - 0x01010101u) ^ (~lo7 & H);  // bytewise x - 1 mod 256
        const uint32_t hi5 = ((hi7 & ~H) + 0x01010101u) ^ (hi7 & H);  // bytewise x + 1 mod 256
        mn7 = min_u16x2(min_u16x2(mn7, prmt(lo7, 0u, 0x4240u)), prmt(lo7, 0u, 0x4341u));
        mx7 = max_u16x2(max_u16x2(mx7, prmt(hi7, 0u, 0x4240u)), prmt(hi7, 0u, 0x4341u));
        mn5 = min_u16x2(min_u16x2(mn5, prmt(lo5, 0u, 0x4240u)), prmt(lo5, 0u, 0x4341u));
        mx5 = max_u16x2(max_u16x2(mx5, prmt(hi5, 0u, 0x4240u)), prmt(hi5, 0u, 0x4341u));
    }
    int min7 = (int)min(mn7 & 0xFFFFu, mn7 >> 16), max7 = (int)max(mx7 & 0xFFFFu, mx7 >> 16);
    int min5 = min((int)min(mn5 & 0xFFFFu, mn5 >> 16) + 1, 255);
    const int m5 = (int)max(mx5 & 0xFFFFu, mx5 >> 16);
    int max5 = m5 > 0 ? m5 - 1 : 0;
    if (min5 > max5) min5 = max5;
    if (min7 > max7) min7 = max7;
    fix_range(min5, max5, 5);
    fix_range(min7, max7, 7);
    uint32_t c5[8], c7[8];
    c5[0] = (uint32_t)min5; c5[1] = (uint32_t)max5;
#pragma unroll
    for (int i = 1; i < 5; ++i) c5[1 + i] = (uint32_t)(((5 - i) * min5 + i * max5) / 5);
    c5[6] = 0; c5[7] = 255;
    // codes7[0..2] are min5/max5 (alpha.rs:237-239), the rest span min7..max7
    c7[0] = (uint32_t)min5; c7[1] = (uint32_t)max5;
#pragma unroll
    for (int i = 1; i < 7; ++i) c7[1 + i] = (uint32_t)(((7 - i) * min7 + i * max7) / 7);
    uint32_t i5[4], i7[4];
    // errors compared without their common x^2 part
    const int e5 = fit_book(v, vm, make_book5((uint32_t)min5, (uint32_t)max5, c5), i5);
    const int e7 = fit_book(v, vm, make_book7((uint32_t)min5, (uint32_t)max5, c7), i7);
    uint32_t out[4];
    if (e5 <= e7) {
        // write_alpha_block5: a0 > a1 cannot occur after fix_range; kept for fidelity
        if (min5 > max5) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                uint32_t w = i5[r], o = 0;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    uint32_t x = (w >> (8 * c)) & 0xFFu;
                    x = x == 0 ? 1u : x == 1 ? 0u : (x <= 5 ? 7u - x : x);
                    o |= x << (8 * c);
                }
                out[r] = o;
            }
            return write_alpha_block((uint32_t)max5, (uint32_t)min5, out);
        }
        return write_alpha_block((uint32_t)min5, (uint32_t)max5, i5);
    }
    // write_alpha_block7: min7 < max7 always holds here; 0<->1, x -> 9-x is (9-x)&7
    if (min7 < max7) {
#pragma unroll
        for (int r = 0; r < 4; ++r) out[r] = (0x09090909u - i7[r]) & 0x07070707u;
        return write_alpha_block((uint32_t)max7, (uint32_t)min7, out);
    }
    return write_alpha_block((uint32_t)min7, (uint32_t)max7, i7);
}

// Interior blocks (all 16 pixels valid, the common case) take the form
// without per-pixel masks; the bytes are the same either way.
__device__ __forceinline__ uint2 encode_bc3_alpha(const uint32_t (&v)[4], uint32_t mask) {
    return mask == 0xFFFFu ? encode_bc3_alpha_t<true>(v, mask) : encode_bc3_alpha_t<false>(v, mask);
}

// Gather one byte channel of 16 RGBA8 pixels into 4 packed words.
__device__ __forceinline__ void channel_words(const uint32_t (&px)[16], int ch, uint32_t (&v)[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int s = 8 * ch;
        v[r] = ((px[4 * r] >> s) & 0xFFu) | (((px[4 * r + 1] >> s) & 0xFFu) << 8) |
               (((px[4 * r + 2] >> s) & 0xFFu) << 16) | (((px[4 * r + 3] >> s) & 0xFFu) << 24);
    }
}

}  // namespace tx
