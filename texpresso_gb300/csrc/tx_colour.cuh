// tx_colour.cuh -- per-block device code for BC1/BC2/BC3 colour endpoints and
// the BC2/BC3 alpha halves, shared by the single-texture kernels (tx_colour.cu)
// and the persistent batch kernel (tx_batch.cu).
//
// Two execution shapes:
//   thread-per-block  ColourSet, SingleColourFit and RangeFit are short and
//                     branch-light; a thread owns a block and 32 neighbouring
//                     blocks load as four coalesced 512-byte rows.
//   team-per-block    ClusterFit: a team of TEAM lanes (16 or 32) owns a block.
//                     Lane p owns pixel p for ColourSet; the candidates (967
//                     least-squares fits at 16 colours) are spread over the
//                     team: each gets a lower bound of its error, only those
//                     the bound cannot exclude get the reference's exact error
//                     (see cand_bound), and the lexicographic minimum on (error,
//                     position in the reference's loop order) selects exactly
//                     the candidate the sequential "first strictly smaller
//                     error" loop selects.
// Both reproduce the reference's f32 operation order (see tx_device.cuh).
// The constant tables are TU-local: every translation unit that includes this
// header uploads its own copy with upload_tables_this_tu().
#pragma once
#include "tx_device.cuh"

namespace tx {

// Single-colour tables (lib/src/colourfit/single_lut.rs): [table][target][index]
// packed start | end << 8 | error << 16.  Tables: 0 = 5_3, 1 = 6_3, 2 = 5_4, 3 = 6_4.
static __constant__ uint32_t c_lut[4][256][2];

// ClusterFit candidate lists.  Entry bits: 0-3 i (offset of S(0,i)),
// 4-11 offset of S(i,j), 12-19 offset of S(j,k) (compress4 only),
// 20-29 rank of (i,j[,k]) in the reference's loop order at 16 colours, so
// comparing entries compares loop positions.
// Entries are sorted so that the first N[n] are exactly the candidates of an
// n-colour set (those with max(i+1, j, k) <= n).
constexpr int kCand4 = 967, kCand3 = 151;
static __device__ uint32_t g_cand[kCand4 + 1 + kCand3 + 1];
static __constant__ uint32_t c_ncand4[17];
static __constant__ uint32_t c_ncand3[17];
// Positions, in the list an n-colour set uses, of its candidates with every
// point in one cluster: compress4 (0,0,n) and (0,n,n), compress3 (0,n).
static __constant__ uint16_t c_one4[17][2];
static __constant__ uint16_t c_one3[17];
// The same candidates in the reference's loop order (i, j, k nested), used for
// 16-colour sets: a round of consecutive candidates then mostly shares S(0,i)
// and S(i,j) and reads S(j,k) at consecutive addresses.
static __device__ uint32_t g_cand16[kCand4 + 1 + kCand3 + 1];
// Lower-bound terms (F1, r, C, S offsets) of the g_cand16 candidates of a
// 16-colour set whose weights are all exactly 1 (the w lanes of the partial
// sums are then the counts i, j-i, k-j), from the reference's f32 alpha2,
// beta2, alphabeta (see unit_terms and unit_bound).  The w lane holds the
// bits i | S(i,j) << 8 | S(j,k) << 16 (table offsets, one byte each).
static __device__ float4 g_ub4[kCand4 + 1];
static __device__ float4 g_ub3[kCand3 + 1];
// unorm8(v) for every byte v and sqrt(n) for n <= 16 (filled by k_unorm_tables
// with the same correctly rounded division and square root as the kernels).
static __device__ float g_unorm8[256];
static __device__ float g_sqrt_count[17];

// Partial-sum table S(a,b), 0 <= a <= b <= 16, stored as the upper triangle
// row by row: S(a,b) at tri_idx(a,b) (153 entries).
__host__ __device__ constexpr int tri_idx(int a, int b) { return a * (33 - a) / 2 + b; }
constexpr int kTri = tri_idx(16, 16) + 1;

// ===========================================================================
// Shared pieces

struct Single {
    uint32_t err;
    float s[3], e[3];
    uint32_t index;  // 0 or 2
};

// SingleColourFit::compute_endpoints (single.rs:58-106).
__device__ __forceinline__ Single single_endpoints(const int (&col)[3], int t0, int t1, int t2) {
    Single r;
    r.err = 0xFFFFFFFFu;
    r.index = 0;
    r.s[0] = r.s[1] = r.s[2] = 0.0f;
    r.e[0] = r.e[1] = r.e[2] = 0.0f;
    const int tb[3] = {t0, t1, t2};
#pragma unroll
    for (int index = 0; index < 2; ++index) {
        uint32_t src[3], err = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            src[c] = c_lut[tb[c]][col[c]][index];
            const uint32_t d = (src[c] >> 16) & 0xFFu;
            err += d * d;
        }
        if (err < r.err) {
            r.s[0] = div_rn((float)(src[0] & 0xFFu), 31.0f);
            r.s[1] = div_rn((float)(src[1] & 0xFFu), 63.0f);
            r.s[2] = div_rn((float)(src[2] & 0xFFu), 31.0f);
            r.e[0] = div_rn((float)((src[0] >> 8) & 0xFFu), 31.0f);
            r.e[1] = div_rn((float)((src[1] >> 8) & 0xFFu), 63.0f);
            r.e[2] = div_rn((float)((src[2] >> 8) & 0xFFu), 31.0f);
            r.index = 2u * (uint32_t)index;
            r.err = err;
        }
    }
    return r;
}

// 2-bit index word for "every valid pixel takes `index`, excluded pixels 3".
__device__ __forceinline__ uint32_t uniform_indices(uint32_t valid16, uint32_t index) {
    uint32_t w = 0;
#pragma unroll
    for (int p = 0; p < 16; ++p) w |= (((valid16 >> p) & 1u) ? index : 3u) << (2 * p);
    return w;
}

// SingleColourFit + ColourFit::compress (colourfit.rs:44-60) given the colour.
template <int FMT>
__device__ __forceinline__ uint2 single_fit(const int (&col)[3], uint32_t valid16, bool transparent) {
    uint32_t best_err = 0xFFFFFFFFu;
    uint2 best = make_uint2(0u, 0u);
    if (FMT == BC1) {
        const Single f = single_endpoints(col, 0, 1, 0);  // LOOKUP_5_3, 6_3, 5_3
        if (f.err < best_err) {
            best = write3(pack_565(f.s[0], f.s[1], f.s[2]), pack_565(f.e[0], f.e[1], f.e[2]),
                          uniform_indices(valid16, f.index));
            best_err = f.err;
        }
    }
    if (FMT != BC1 || !transparent) {
        const Single f = single_endpoints(col, 2, 3, 2);  // LOOKUP_5_4, 6_4, 5_4
        if (f.err < best_err) {
            best = write4(pack_565(f.s[0], f.s[1], f.s[2]), pack_565(f.e[0], f.e[1], f.e[2]),
                          uniform_indices(valid16, f.index));
        }
    }
    return best;
}

// Sym3x3::principle_component (math.rs:75-97); only lanes x,y,z matter.
__device__ __forceinline__ void principle_component(const float (&m)[6], float (&v)[3]) {
    float vx = 1.0f, vy = 1.0f, vz = 1.0f;
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float wx = m[0] * vx, wy = m[1] * vx, wz = m[2] * vx;
        wx = m[1] * vy + wx; wy = m[3] * vy + wy; wz = m[4] * vy + wz;
        wx = m[2] * vz + wx; wy = m[4] * vz + wy; wz = m[5] * vz + wz;
        const float a = fmaxf(wx, fmaxf(wy, wz));
        const float r = rcp_rn(a);
        vx = wx * r; vy = wy * r; vz = wz * r;
    }
    v[0] = vx; v[1] = vy; v[2] = vz;
}

// Clamp to [0,1] and snap to the 5:6:5 grid (range.rs:87-98, cluster.rs:206-210).
__device__ __forceinline__ float snap(float x, float grid, float gridrcp) {
    x = fminf(1.0f, fmaxf(0.0f, x));
    return truncf(grid * x + 0.5f) * gridrcp;
}

__device__ __forceinline__ uint32_t u8_of(uint32_t px, int c) { return (px >> (8 * c)) & 0xFFu; }

// ===========================================================================
// k_range: one thread per block

// Per-thread point store for the thread-per-block path: pixel i of thread t
// lives at pts[i * stride + t] as (x, y, z, weight), so a warp's loads of one
// pixel are 512 contiguous bytes (no bank conflicts) and the fit keeps only
// accumulators in registers.
struct PointCol {
    float4 *base;
    int stride;
    __device__ __forceinline__ float4 &operator[](int i) const { return base[i * stride]; }
};

// The duplicate search of ColourSet::new (colourset.rs:82-102) for one block:
// each pixel's point is the first pixel with its key, and a point's pixel
// count is one plus the later pixels that join it.  res (4 words) receives
// byte p = pixel p's point index | (count - 1) << 4 (the count half is kept
// for points only).  Keys: the RGB of a valid pixel, or 0x01000000 | p for a
// pixel that is not (so it matches nothing).
__device__ __forceinline__ void colour_dedup(const uint32_t (&key)[16], uint32_t (&res)[4]) {
    // One comparison per pair j < i: it moves i's point down to j (the last
    // assignment, at the smallest j, wins) and counts i as a later pixel of
    // j's colour in the high nibble of byte j.  Every shift is a constant.
    uint32_t cnt[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int w = 0; w < 4; ++w) res[w] = 0u;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        uint32_t r = (uint32_t)i;
#pragma unroll
        for (int j = i - 1; j >= 0; --j) {
            const bool e = key[j] == key[i];
            r = e ? (uint32_t)j : r;
            cnt[j >> 2] += e ? (0x10u << (8 * (j & 3))) : 0u;
        }
        res[i >> 2] |= r << (8 * (i & 3));
    }
#pragma unroll
    for (int w = 0; w < 4; ++w) res[w] |= cnt[w];
}

// Point index and (pixel count - 1) of pixel i from colour_dedup's bytes.
__device__ __forceinline__ uint32_t dd_rep(const uint32_t (&res)[4], int i) { return (res[i >> 2] >> (8 * (i & 3))) & 0xFu; }
__device__ __forceinline__ uint32_t dd_dup(const uint32_t (&res)[4], int i) {
    return (res[i >> 2] >> (8 * (i & 3) + 4)) & 0xFu;
}

// px is overwritten with the colour-set keys (the RGB bytes of every valid
// pixel are kept; alpha is not needed after the packed copy below), so the
// pixels and the keys never occupy registers at the same time.
template <int FMT>
__device__ __forceinline__ uint2 colour_range_thread(uint32_t (&px)[16], uint32_t inb,
                                                     const DevParams &prm, const float *s_unorm,
                                                     const float *s_sqrt, const PointCol &pt) {
    // ColourSet (colourset.rs:35-112), pixel-indexed: a "point" is the first
    // pixel of its colour, and pixel order is point order.
    uint32_t tbits = 0;
    if (FMT == BC1) {
#pragma unroll
        for (int i = 0; i < 16; ++i) tbits |= ((px[i] >> 31) ^ 1u) << i;
        tbits &= inb;
    }
    const uint32_t valid = inb & ~tbits;
    const bool transparent = tbits != 0;
    uint32_t a4[4];  // alpha of pixel 4r + c at byte c of a4[r] (alpha weighting only)
    if (prm.alpha_weighted) channel_words(px, 3, a4);
#pragma unroll
    for (int i = 0; i < 16; ++i) px[i] = ((valid >> i) & 1u) ? (px[i] & 0xFFFFFFu) : (0x01000000u | (uint32_t)i);
    uint32_t dd[4];  // byte p: pixel p's point index | (its colour's pixel count - 1) << 4
    colour_dedup(px, dd);
    // a valid pixel that is its own point starts a new point (excluded pixels
    // match nothing, so they are their own "point" too and are masked out)
    uint32_t newbits = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        const uint32_t eq = bytes_eq(dd[w] & 0x0F0F0F0Fu, 0x03020100u + 0x04040404u * (uint32_t)w);
        newbits |= (((eq & 0x08040201u) * 0x01010101u) >> 24) << (4 * w);
    }
    newbits &= valid;
    const int count = __popc(newbits);

    if (count == 1) {
        uint32_t rgb = 0;
#pragma unroll
        for (int i = 0; i < 16; ++i) rgb |= ((valid >> i) & 1u) ? px[i] : 0u;
        int col[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) col[c] = f32_to_i32_clamped(s_unorm[u8_of(rgb, c)] * 255.0f, 255);
        return single_fit<FMT>(col, valid, transparent);
    }

    // Points and weights.  Pixels that are not points get weight exactly 0,
    // which makes their terms +-0 in every ordered sum below.  Those sums start
    // at +0 and add non-negative values (total, centroid) or can only reach
    // zero as +0 (round-to-nearest x + (-x) = +0), so they are never -0 and
    // adding +-0 leaves them unchanged: the sums equal the reference's sums
    // over points.
    if (!prm.alpha_weighted) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float w = ((newbits >> i) & 1u) ? s_sqrt[1 + (int)dd_dup(dd, i)] : 0.0f;
            pt[i] = make_float4(s_unorm[u8_of(px[i], 0)], s_unorm[u8_of(px[i], 1)], s_unorm[u8_of(px[i], 2)], w);
        }
    } else {
        // alpha weights (colourset.rs:69-74, :94-97): every valid pixel adds
        // (a + 1) / 256 to its point's weight in pixel order, the point's own
        // pixel first (0 + w = w); an excluded pixel adds +0 to its own slot,
        // which stays +0.  Then sqrt for the points.
#pragma unroll
        for (int j = 0; j < 16; ++j)
            pt[j] = make_float4(s_unorm[u8_of(px[j], 0)], s_unorm[u8_of(px[j], 1)], s_unorm[u8_of(px[j], 2)], 0.0f);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float wa = ((valid >> i) & 1u)
                                 ? (float)(((a4[i >> 2] >> (8 * (i & 3))) & 0xFFu) + 1u) * (1.0f / 256.0f)
                                 : 0.0f;
            float &w = pt[(int)dd_rep(dd, i)].w;
            w = w + wa;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if ((newbits >> j) & 1u) pt[j].w = sqrt_rn(pt[j].w);
    }

    // Sym3x3::weighted_covariance (math.rs:44-73)
    float total = 0.0f, cx = 0.0f, cy = 0.0f, cz = 0.0f;
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
        const float4 q = pt[i];
        total = total + q.w;
        cx = cx + q.x * q.w; cy = cy + q.y * q.w; cz = cz + q.z * q.w;
    }
    if (total > FLT_EPSILON) { cx = div_rn(cx, total); cy = div_rn(cy, total); cz = div_rn(cz, total); }
    float m[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
        const float4 q = pt[i];
        const float ax = q.x - cx, ay = q.y - cy, az = q.z - cz;
        const float bx = ax * q.w, by = ay * q.w, bz = az * q.w;
        m[0] += ax * bx; m[1] += ax * by; m[2] += ax * bz;
        m[3] += ay * by; m[4] += ay * bz; m[5] += az * bz;
    }
    float axis[3];
    principle_component(m, axis);

    // RangeFit::new (range.rs:44-101): the first point starts both ends; a later
    // point moves start on a strictly smaller dot, else end on a strictly larger one
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, e0 = 0.0f, e1 = 0.0f, e2 = 0.0f;
    if (count > 0) {
        bool seen = false;
        float mn = 0.0f, mx = 0.0f;
        int si = 0, ei = 0;
#pragma unroll 4
        for (int i = 0; i < 16; ++i) {
            const float4 q = pt[i];
            const bool p = (newbits >> i) & 1u;
            const float d = q.x * axis[0] + q.y * axis[1] + q.z * axis[2];
            const bool first = p && !seen;
            const bool lo = first || (p && d < mn);
            const bool hi = first || (p && !(d < mn) && d > mx);
            si = lo ? i : si; mn = lo ? d : mn;
            ei = hi ? i : ei; mx = hi ? d : mx;
            seen = seen || p;
        }
        const float4 qs = pt[si], qe = pt[ei];
        s0 = qs.x; s1 = qs.y; s2 = qs.z;
        e0 = qe.x; e1 = qe.y; e2 = qe.z;
    }
    s0 = snap(s0, 31.0f, 1.0f / 31.0f); s1 = snap(s1, 63.0f, 1.0f / 63.0f); s2 = snap(s2, 31.0f, 1.0f / 31.0f);
    e0 = snap(e0, 31.0f, 1.0f / 31.0f); e1 = snap(e1, 63.0f, 1.0f / 63.0f); e2 = snap(e2, 31.0f, 1.0f / 31.0f);

    const float w0 = prm.w[0], w1 = prm.w[1], w2 = prm.w[2];
    float best_err = FLT_MAX;
    uint2 best = make_uint2(0u, 0u);

    // compression_helper (range.rs:103-143) over a codebook of nc codes.  The
    // error sum adds +0 for pixels that are not points (it starts at +0 and
    // its terms are non-negative).
    // The weighted differences w (x - c) of codes (0,1) and (2,3) are formed
    // in pairs by the paired f32 operations add2_rn / mul2_rn (each lane the
    // IEEE operation of the scalar form, x - c being x + (-c); an add followed
    // by a multiply leaves nothing to fuse).  The squares and their sum stay
    // scalar: a paired multiply followed by a paired add was contracted into
    // a fused multiply-add even when written with .rn, which changes the
    // rounding.  So every distance is the reference's
    // ((w0 (x - cr))^2 + (w1 (y - cg))^2) + (w2 (z - cb))^2.
    const float2 W0 = make_float2(w0, w0), W1 = make_float2(w1, w1), W2 = make_float2(w2, w2);
    auto helper = [&](const float (&cr)[4], const float (&cg)[4], const float (&cb)[4], int nc,
                      uint32_t &indices) -> bool {
        const float2 nr01 = make_float2(-cr[0], -cr[1]), nr23 = make_float2(-cr[2], -cr[3]);
        const float2 ng01 = make_float2(-cg[0], -cg[1]), ng23 = make_float2(-cg[2], -cg[3]);
        const float2 nb01 = make_float2(-cb[0], -cb[1]), nb23 = make_float2(-cb[2], -cb[3]);
        uint32_t closest = 0;
        float err = 0.0f;
#pragma unroll 4
        for (int i = 0; i < 16; ++i) {
            const float4 q = pt[i];
            const float2 X = make_float2(q.x, q.x), Y = make_float2(q.y, q.y), Z = make_float2(q.z, q.z);
            const float2 dx01 = mul2_rn(W0, add2_rn(X, nr01)), dx23 = mul2_rn(W0, add2_rn(X, nr23));
            const float2 dy01 = mul2_rn(W1, add2_rn(Y, ng01)), dy23 = mul2_rn(W1, add2_rn(Y, ng23));
            const float2 dz01 = mul2_rn(W2, add2_rn(Z, nb01)), dz23 = mul2_rn(W2, add2_rn(Z, nb23));
            const float dx[4] = {dx01.x, dx01.y, dx23.x, dx23.y}, dy[4] = {dy01.x, dy01.y, dy23.x, dy23.y};
            const float dz[4] = {dz01.x, dz01.y, dz23.x, dz23.y};
            float d[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) d[j] = dx[j] * dx[j] + dy[j] * dy[j] + dz[j] * dz[j];
            float dist = FLT_MAX;
            uint32_t idx = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (j < nc) {
                    idx = d[j] < dist ? (uint32_t)j : idx;
                    dist = d[j] < dist ? d[j] : dist;
                }
            }
            closest |= idx << (2 * i);
            err = err + (((newbits >> i) & 1u) ? dist : 0.0f);
        }
        if (err < best_err) {
            // remap_indices (colourset.rs:130-141); with 16 distinct valid
            // pixels every pixel is its own point and the map is the identity
            uint32_t out = closest;
            if (newbits != 0xFFFFu) {
                out = 0;
#pragma unroll
                for (int p = 0; p < 16; ++p) {
                    const uint32_t r = dd_rep(dd, p);
                    const uint32_t v = ((valid >> p) & 1u) ? ((closest >> (2 * r)) & 3u) : 3u;
                    out |= v << (2 * p);
                }
            }
            indices = out;
            best_err = err;
            return true;
        }
        return false;
    };

    const uint32_t a565 = pack_565(s0, s1, s2), b565 = pack_565(e0, e1, e2);
    if (FMT == BC1) {
        const float cr[4] = {s0, e0, s0 * 0.5f + e0 * 0.5f, 0.0f};
        const float cg[4] = {s1, e1, s1 * 0.5f + e1 * 0.5f, 0.0f};
        const float cb[4] = {s2, e2, s2 * 0.5f + e2 * 0.5f, 0.0f};
        uint32_t idx;
        if (helper(cr, cg, cb, 3, idx)) best = write3(a565, b565, idx);
    }
    if (FMT != BC1 || !transparent) {
        const float c23 = 2.0f / 3.0f, c13 = 1.0f / 3.0f;
        const float cr[4] = {s0, e0, s0 * c23 + e0 * c13, s0 * c13 + e0 * c23};
        const float cg[4] = {s1, e1, s1 * c23 + e1 * c13, s1 * c13 + e1 * c23};
        const float cb[4] = {s2, e2, s2 * c23 + e2 * c13, s2 * c13 + e2 * c23};
        uint32_t idx;
        if (helper(cr, cg, cb, 4, idx)) best = write4(a565, b565, idx);
    }
    return best;
}

__device__ __forceinline__ void init_unorm_tables(float *s_unorm, float *s_sqrt) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_unorm[i] = unorm8((uint32_t)i);
    if (threadIdx.x < 17) s_sqrt[threadIdx.x] = sqrt_rn((float)threadIdx.x);
    __syncthreads();
}

// The same tables in global memory (one CTA of 256 threads).
static __global__ void k_unorm_tables() {
    g_unorm8[threadIdx.x] = unorm8(threadIdx.x);
    if (threadIdx.x < 17) g_sqrt_count[threadIdx.x] = sqrt_rn((float)threadIdx.x);
}

// ===========================================================================
// k_cluster: one team per block

template <int TEAM>
struct Team {
    unsigned mask;
    int lane;
    int base;
    __device__ __forceinline__ Team() {
        const int wl = threadIdx.x & 31;
        lane = wl & (TEAM - 1);
        base = wl & ~(TEAM - 1);
        mask = (TEAM == 32) ? 0xFFFFFFFFu : (0xFFFFu << base);
    }
    __device__ __forceinline__ unsigned ballot(bool p) const {
        const unsigned b = __ballot_sync(mask, p);
        return (TEAM == 32) ? b : ((b >> base) & 0xFFFFu);
    }
    __device__ __forceinline__ bool all(bool p) const { return __all_sync(mask, p); }
    template <class T> __device__ __forceinline__ T shfl(T v, int src) const { return __shfl_sync(mask, v, src, TEAM); }
    template <class T> __device__ __forceinline__ T shfl_xor(T v, int m) const { return __shfl_xor_sync(mask, v, m, TEAM); }
    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ unsigned match(uint32_t key) const {
        const unsigned m = __match_any_sync(mask, key);
        return (TEAM == 32) ? m : ((m >> base) & 0xFFFFu);
    }
};

struct __align__(16) TeamSmem {
    float4 S[kTri + 3];     // S(a,b) running sums at tri_idx(a,b) (+pad)
    union {                 // lifetimes do not overlap within an iteration:
        float LB[kCand4 + 1];   // candidate lower bounds, then the survivor queue
        struct {
            float4 PW[16];      // points_weights in the current ordering
            uint32_t D[16];     // sort keys of the dot products
        };
    };
    float P[4][16];         // x, y, z, weight of each point, point order
    uint32_t hist[8][4];    // orderings of earlier iterations (16 bytes each)
};

// Sym3x3::principle_component (math.rs:75-97) for a team: lane c < 3 forms
// component c of each product M v in the reference's order (row 0 times vx,
// then row 1 times vy added, then row 2 times vz), and every lane takes the
// three components by shuffle for the max and the scaling.
template <int TEAM>
__device__ __forceinline__ void principle_component_team(const Team<TEAM> &tm, const float (&m)[6], float (&v)[3]) {
    const int c = tm.lane < 3 ? tm.lane : 0;
    const float a0 = c == 0 ? m[0] : (c == 1 ? m[1] : m[2]);
    const float a1 = c == 0 ? m[1] : (c == 1 ? m[3] : m[4]);
    const float a2 = c == 0 ? m[2] : (c == 1 ? m[4] : m[5]);
    float vx = 1.0f, vy = 1.0f, vz = 1.0f;
#pragma unroll 1
    for (int it = 0; it < 8; ++it) {
        float w = a0 * vx;
        w = a1 * vy + w;
        w = a2 * vz + w;
        const float wx = tm.shfl(w, 0), wy = tm.shfl(w, 1), wz = tm.shfl(w, 2);
        const float r = rcp_rn(fmaxf(wx, fmaxf(wy, wz)));
        vx = wx * r; vy = wy * r; vz = wz * r;
    }
    v[0] = vx; v[1] = vy; v[2] = vz;
}

// Sort key of cluster.rs:90-97 as an unsigned integer: finite values keep
// their order (-0 and +0 tie), every non-finite value ties after all finite
// ones.  Comparing keys is comparing with fcmp.
__device__ __forceinline__ uint32_t dps_key(float x) {
    if (!isfinite(x)) return 0xFFFFFFFFu;
    const uint32_t u = (uint32_t)__float_as_int(x + 0.0f);  // -0 -> +0
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// min(1, max(0, fl(a * b))) in one instruction: mul.rn with .sat clamps the
// rounded product to [0, 1] and turns NaN into +0, as f32::max/min do in
// cluster.rs:207-208 (max(0, NaN) = 0).
__device__ __forceinline__ float mul_sat(float a, float b) {
    float d;
    asm("mul.rn.sat.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}

// Snap a value already clamped to [0, 1] to the grid (cluster.rs:209-210).
__device__ __forceinline__ float snap01(float x, float grid, float gridrcp) {
    return truncf(grid * x + 0.5f) * gridrcp;
}

__device__ __forceinline__ uint8_t hist_get(const TeamSmem &sm, int it, int m) {
    return reinterpret_cast<const uint8_t *>(sm.hist[it])[m];
}

// Weight-lane terms of one compress4 candidate (cluster.rs:320-335).
__device__ __forceinline__ float4 wterms4(float p0w, float p1w, float p2w, float xsw) {
    const float c19 = 1.0f / 9.0f, c49 = 4.0f / 9.0f, c29 = 2.0f / 9.0f;
    const float p3w = xsw - p2w - p1w - p0w;
    const float alpha2 = p2w * c19 + (p1w * c49 + p0w);
    const float beta2 = p1w * c19 + (p2w * c49 + p3w);
    const float ab = c29 * (p1w + p2w);
    return make_float4(alpha2, beta2, ab, rcp_rn((alpha2 * beta2) - ab * ab));
}

// Weight-lane terms of one compress3 candidate (cluster.rs:189-202).  The
// products part1 * (.5, .25) are exact, so each sum is one fused op.
__device__ __forceinline__ float4 wterms3(float p0w, float p1w, float xsw) {
    const float p2w = xsw - p1w - p0w;
    const float alpha2 = __fmaf_rn(p1w, 0.25f, p0w);
    const float beta2 = __fmaf_rn(p1w, 0.25f, p2w);
    const float ab = p1w * 0.25f;
    return make_float4(alpha2, beta2, ab, rcp_rn((alpha2 * beta2) - ab * ab));
}

// Endpoint fit and error of one candidate given its x/y/z sums ax, bx and its
// weight-lane terms wt (cluster.rs:200-220, :333-353).
template <bool WANT_AB>
__device__ __forceinline__ float fit_error(const float (&ax)[3], const float (&bx)[3], const float4 wt,
                                           const float (&cw)[3], float (&ea)[3], float (&eb)[3]) {
    const float alpha2 = wt.x, beta2 = wt.y, ab = wt.z, factor = wt.w;
    const float grid[3] = {31.0f, 63.0f, 31.0f};
    const float gridrcp[3] = {1.0f / 31.0f, 1.0f / 63.0f, 1.0f / 31.0f};
    float e5[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a = snap01(mul_sat((ax[c] * beta2) - bx[c] * ab, factor), grid[c], gridrcp[c]);
        const float b = snap01(mul_sat((bx[c] * alpha2) - ax[c] * ab, factor), grid[c], gridrcp[c]);
        const float e1 = (a * a) * alpha2 + (b * b * beta2);
        const float e2 = (a * b * ab) - a * ax[c];
        const float e3 = e2 - b * bx[c];
        const float e4 = __fmaf_rn(2.0f, e3, e1);  // 2*e3 is exact, so this equals fl(fl(2*e3) + e1)
        e5[c] = e4 * cw[c];
        if (WANT_AB) { ea[c] = a; eb[c] = b; }
    }
    return e5[0] + e5[1] + e5[2];
}

// One compress4 candidate (cluster.rs:320-353); wt = wterms4(...) of its w lanes.
template <bool WANT_AB>
__device__ __forceinline__ float eval4(const float4 p0, const float4 p1, const float4 p2, const float4 xs,
                                       const float4 wt, const float (&cw)[3], float (&ea)[3], float (&eb)[3]) {
    const float c13 = 1.0f / 3.0f, c23 = 2.0f / 3.0f;
    const float p3x = xs.x - p2.x - p1.x - p0.x;
    const float p3y = xs.y - p2.y - p1.y - p0.y;
    const float p3z = xs.z - p2.z - p1.z - p0.z;
    const float ax[3] = {p2.x * c13 + (p1.x * c23 + p0.x), p2.y * c13 + (p1.y * c23 + p0.y),
                         p2.z * c13 + (p1.z * c23 + p0.z)};
    const float bx[3] = {p1.x * c13 + (p2.x * c23 + p3x), p1.y * c13 + (p2.y * c23 + p3y),
                         p1.z * c13 + (p2.z * c23 + p3z)};
    return fit_error<WANT_AB>(ax, bx, wt, cw, ea, eb);
}

// One compress3 candidate (cluster.rs:189-220); wt = wterms3(...) of its w lanes.
template <bool WANT_AB>
__device__ __forceinline__ float eval3(const float4 p0, const float4 p1, const float4 xs, const float4 wt,
                                       const float (&cw)[3], float (&ea)[3], float (&eb)[3]) {
    const float p2x = xs.x - p1.x - p0.x, p2y = xs.y - p1.y - p0.y, p2z = xs.z - p1.z - p0.z;
    const float ax[3] = {__fmaf_rn(p1.x, 0.5f, p0.x), __fmaf_rn(p1.y, 0.5f, p0.y), __fmaf_rn(p1.z, 0.5f, p0.z)};
    const float bx[3] = {__fmaf_rn(p1.x, 0.5f, p2x), __fmaf_rn(p1.y, 0.5f, p2y), __fmaf_rn(p1.z, 0.5f, p2z)};
    return fit_error<WANT_AB>(ax, bx, wt, cw, ea, eb);
}

// Decode (i, j, k) from a candidate entry.
__host__ __device__ __forceinline__ void decode_entry(uint32_t e, int &i, int &j, int &k) {
    i = (int)(e & 0xFu);
    j = (int)((e >> 4) & 0xFFu) - tri_idx(i, 0);
    k = (int)((e >> 12) & 0xFFu) - tri_idx(j, 0);
}

// ---------------------------------------------------------------------------
// Candidate pruning.  For a candidate with weight-lane terms alpha, beta,
// gamma (> 0 definite) and per-channel sums ax, bx, the reference's error at
// any endpoints (a, b) is  sum_c w_c Q_c(a_c, b_c)  with
//     Q(a, b) = alpha a^2 + beta b^2 + 2 gamma a b - 2 a ax - 2 b bx
// (cluster.rs:345-353, evaluated in f32).  Q is minimised over all real (a, b)
// by the unclamped least-squares endpoints, where it equals
//     -q,  q = (beta ax^2 - 2 gamma ax bx + alpha bx^2) / det,
// so no clamping or grid snapping can bring the error below -sum_c w_c q_c.
// With bx = X - ax (X_c the channel sums) and A = alpha + beta + 2 gamma,
// B = alpha + gamma, the numerator summed over channels is
//     sum_c w_c q_c det = A sum_c w_c ax_c^2 - 2B sum_c w_c X_c ax_c + alpha Z,
// Z = sum_c w_c X_c^2 being the same for every candidate of the block.  The
// bound is evaluated in that form with cheaper arithmetic than the reference
// (FMA, an approximate reciprocal), and the difference to the reference's f32
// error is covered by a margin (weights w_c >= 0, all sums non-negative,
// W = weight sum, u = 2^-24):
//   * rounding of the reference's own error evaluation, and using f32
//     weight-lane terms that differ from its by a few ulps: <= 36 u W sum(w);
//   * our ax (and X - ax) within 16 u X of the reference's ax, bx, moving the
//     minimum by at most 32 u X (|A*| + |B*|) <= 32 u f W X^2, plus rounding of
//     the three sums, their combination and f: <= 26 u f W Z;
// so  E_ref >= -f (sum_c w_c q_c det + Kb) - eps1  with  Kb = 2^-17 W Z and
// eps1 = 2^-17 W sum w_c (128 u, about twice the derived terms).
// A candidate whose bound exceeds an error some candidate actually reaches
// can neither win nor tie, so the exact sweep only needs the others.  The
// result is the reference's choice bit for bit; only the work changes.

// Bound terms (A, -2B, alpha, 1/det) from the w lanes of the partial sums, for
// blocks whose weights are not all 1 (no table entry applies).
template <int NC>
__device__ __forceinline__ float4 lb_terms(float p0w, float p1w, float p2w, float xsw) {
    float al, be, g2;
    if (NC == 4) {
        const float p3w = xsw - p0w - p1w - p2w;
        al = __fmaf_rn(p2w, 1.0f / 9.0f, __fmaf_rn(p1w, 4.0f / 9.0f, p0w));
        be = __fmaf_rn(p1w, 1.0f / 9.0f, __fmaf_rn(p2w, 4.0f / 9.0f, p3w));
        g2 = (4.0f / 9.0f) * (p1w + p2w);
    } else {
        const float p2r = xsw - p0w - p1w;
        al = __fmaf_rn(p1w, 0.25f, p0w);
        be = __fmaf_rn(p1w, 0.25f, p2r);
        g2 = 0.5f * p1w;
    }
    // det = al*be - g*g with the product g*g split exactly (its rounding error
    // recovered by an FMA), so det carries only the final roundings
    const float g = 0.5f * g2;
    const float gg = g * g;
    const float gerr = __fmaf_rn(g, g, -gg);
    const float det = __fmaf_rn(al, be, -gg) - gerr;
    float f;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"(det));
    return make_float4(al + be + g2, -(2.0f * al + g2), al, det > 0.0f ? f : __int_as_float(0x7fc00000));  // NaN: no bound
}

// Per-block constants of the bound: w_c X_c, Z = sum_c w_c X_c^2, Kb, eps1.
struct BoundBlock {
    float wx[3], z, kb, eps1;
};

__device__ __forceinline__ BoundBlock bound_block(const float4 xs, const float (&cw)[3]) {
    BoundBlock bb;
    bb.wx[0] = cw[0] * xs.x;
    bb.wx[1] = cw[1] * xs.y;
    bb.wx[2] = cw[2] * xs.z;
    float z = 0.0f;
    z = __fmaf_rn(cw[0], xs.x * xs.x, z);
    z = __fmaf_rn(cw[1], xs.y * xs.y, z);
    z = __fmaf_rn(cw[2], xs.z * xs.z, z);
    bb.z = z;
    bb.kb = 7.62939453125e-6f * xs.w * z;                          // 2^-17 W Z
    bb.eps1 = 7.62939453125e-6f * xs.w * (cw[0] + cw[1] + cw[2]);  // 2^-17 W sum w
    return bb;
}

// -f (A sum w ax^2 - 2B sum w X ax + alpha Z + Kb) - eps1 for one candidate;
// lt = (A, -2B, alpha, f).
template <int NC>
__device__ __forceinline__ float cand_bound(const float4 p0, const float4 p1, const float4 p2, const float4 lt,
                                            const float (&cw)[3], const BoundBlock &bb) {
    const float pa[3] = {p0.x, p0.y, p0.z}, pb[3] = {p1.x, p1.y, p1.z}, pc[3] = {p2.x, p2.y, p2.z};
    float ax[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        ax[c] = (NC == 4) ? __fmaf_rn(pc[c], 1.0f / 3.0f, __fmaf_rn(pb[c], 2.0f / 3.0f, pa[c]))
                          : __fmaf_rn(pb[c], 0.5f, pa[c]);
    float s1 = (cw[0] * ax[0]) * ax[0];
    s1 = __fmaf_rn(cw[1] * ax[1], ax[1], s1);
    s1 = __fmaf_rn(cw[2] * ax[2], ax[2], s1);
    float s2 = bb.wx[0] * ax[0];
    s2 = __fmaf_rn(bb.wx[1], ax[1], s2);
    s2 = __fmaf_rn(bb.wx[2], ax[2], s2);
    const float acc = __fmaf_rn(lt.x, s1, __fmaf_rn(lt.y, s2, __fmaf_rn(lt.z, bb.z, bb.kb)));
    return __fmaf_rn(-lt.w, acc, -bb.eps1);  // NaN when there is no bound: the candidate is kept
}

// The same bound for a 16-colour set of weight-1 points (W = 16), with the
// candidate's constants folded into q = (F1, r, C) = (-A f, 2B / A,
// -f (alpha + 2^-13)) (double, rounded once): since
//     -f (A s1 - 2B s2) = F1 sum_c w_c ax_c (ax_c - r X_c)
// and -f (alpha Z + Kb) = C Z (Kb = 2^-17 W Z = 2^-13 Z), the bound is
//     F1 sum_c w_c ax_c (ax_c - r X_c) + C Z - eps1.
// Rounding: A = W exactly, 0 <= r <= 2, so each of the three products is at
// most 2 w_c X_c^2 in size and the sum carries at most ~10 u Z; with the
// rounding of F1, r, C and the two final FMAs that is <= ~17 u f W Z, inside
// the 26 u f W Z budgeted for the general form above.
template <int NC>
__device__ __forceinline__ float unit_bound(const float4 p0, const float4 p1, const float4 p2, const float4 q,
                                            const float4 xs, const float (&cw)[3], const BoundBlock &bb) {
    const float pa[3] = {p0.x, p0.y, p0.z}, pb[3] = {p1.x, p1.y, p1.z}, pc[3] = {p2.x, p2.y, p2.z};
    const float X[3] = {xs.x, xs.y, xs.z};
    float sum = 0.0f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float ax = (NC == 4) ? __fmaf_rn(pc[c], 1.0f / 3.0f, __fmaf_rn(pb[c], 2.0f / 3.0f, pa[c]))
                                   : __fmaf_rn(pb[c], 0.5f, pa[c]);
        const float d = __fmaf_rn(-q.y, X[c], ax);
        sum = c == 0 ? (cw[0] * ax) * d : __fmaf_rn(cw[c] * ax, d, sum);
    }
    return __fmaf_rn(q.x, sum, __fmaf_rn(q.z, bb.z, -bb.eps1));  // NaN when there is no bound
}

// Per-lane best of the candidates a lane evaluated exactly: error, entry and
// endpoints, compared lexicographically on (error, entry).
struct LaneBest {
    float err;
    uint32_t ent;
    float a[3], b[3];
};

// Exact error and endpoints of the candidate entry e (cluster.rs:189-220,
// :320-353), folded into the lane's best.
template <int NC>
__device__ __forceinline__ void eval_candidate(const TeamSmem &sm, uint32_t e, const float4 xs, const float (&cw)[3],
                                               LaneBest &lb) {
    float a[3], b[3], err;
    const float4 p0 = sm.S[e & 0xFu];
    const float4 p1 = sm.S[(e >> 4) & 0xFFu];
    if (NC == 4) {
        const float4 p2 = sm.S[(e >> 12) & 0xFFu];
        err = eval4<true>(p0, p1, p2, xs, wterms4(p0.w, p1.w, p2.w, xs.w), cw, a, b);
    } else {
        err = eval3<true>(p0, p1, xs, wterms3(p0.w, p1.w, xs.w), cw, a, b);
    }
    if (err < lb.err || (err == lb.err && e < lb.ent)) {
        lb.err = err;
        lb.ent = e;
#pragma unroll
        for (int c = 0; c < 3; ++c) { lb.a[c] = a[c]; lb.b[c] = b[c]; }
    }
}

// The ordering along the principal axis is the first ordering of both
// compress3 and compress4 (cluster.rs:78-136 with the same axis and points),
// so compress4 takes it and its partial sums from compress3 when compress3
// built no later ordering over them.
struct SharedOrder {
    bool valid;  // S and hist[0] hold the principal-axis ordering
    int rank;    // this lane's point's position in it
    bool finite; // every dot product was finite
};

// ClusterFit::compress3 / compress4 (cluster.rs:152-417) for one team.
// best_err / best carry the ColourFit state across compress3 -> compress4.
// LEAN (BC1 IterativeClusterFit, whose two passes make the largest kernel and
// whose top stall is instruction fetch) trades unrolling for code size: the
// rank and partial-sum loops are unrolled 4 times instead of 16, and short
// lists go through the survivor sweep instead of a sweep of their own
// (1,557 vs 1,604 us for 2048x2048; the other kernels measured faster
// without these changes).
template <int NC, int TEAM, int NITER, bool LEAN = false>
__device__ __forceinline__ void cluster_pass(const Team<TEAM> &tm, TeamSmem &sm, const uint32_t *tbl, int count,
                                             const float (&principal)[3], const float (&cw)[3], bool prune,
                                             bool valid, int my_point, bool unit16, float &best_err, uint2 &best,
                                             SharedOrder &so) {
    const int lane = tm.lane;
    float run = best_err;
    float ba[3] = {0.0f, 0.0f, 0.0f}, bb[3] = {0.0f, 0.0f, 0.0f};
    uint32_t bentry = 0;
    int bit = 0, best_rank = 0;
    bool best_finite = false;
    float axis[3] = {principal[0], principal[1], principal[2]};
    const uint32_t ncand = (NC == 4) ? c_ncand4[count] : c_ncand3[count];
    float4 xs = make_float4(0.f, 0.f, 0.f, 0.f);

#pragma unroll 1
    for (int it = 0; it < NITER; ++it) {
        // construct_ordering (cluster.rs:78-136)
        int my_rank = 0;
        bool finite;
        if (NITER == 1 && so.valid) {  // (the iterative kernel measured faster rebuilding it)
            my_rank = so.rank;
            finite = so.finite;
        } else {
            float de = FLT_MAX;
            if (lane < count) de = sm.P[0][lane] * axis[0] + sm.P[1][lane] * axis[1] + sm.P[2][lane] * axis[2];
            const uint32_t ke = dps_key(de);
            if (lane < 16) sm.D[lane] = ke;
            tm.sync();
            if (lane < 16) {
                // stable rank: entries with a smaller key, or an equal key earlier
                int rank = 0;
                if (LEAN) {
#pragma unroll 4
                    for (int f = 0; f < 16; ++f) {
                        const uint32_t kf = sm.D[f];
                        rank += (kf < ke || (kf == ke && f < lane)) ? 1 : 0;
                    }
                } else {
#pragma unroll
                    for (int f = 0; f < 16; ++f) {
                        const uint32_t kf = sm.D[f];
                        rank += (kf < ke || (kf == ke && f < lane)) ? 1 : 0;
                    }
                }
                reinterpret_cast<uint8_t *>(sm.hist[it])[rank] = (uint8_t)(lane < count ? lane : 0);
                my_rank = rank;
            }
            // with every dot product finite, positions 0..count-1 hold each point once
            finite = tm.ballot(lane < count && ke == 0xFFFFFFFFu) == 0u;
            tm.sync();
            const int my_ord = (lane < 16) ? hist_get(sm, it, lane) : 0;
            bool repeated = false;
#pragma unroll 1
            for (int t = 0; t < it; ++t) repeated |= tm.all(lane >= 16 || hist_get(sm, t, lane) == my_ord);
            if (repeated) break;
            if (lane < count) {
                const float w = sm.P[3][my_ord];
                sm.PW[lane] = make_float4(sm.P[0][my_ord] * w, sm.P[1][my_ord] * w, sm.P[2][my_ord] * w, 1.0f * w);
            }
            tm.sync();
            // partial sums S(a,b) = pw[a] + ... + pw[b-1], accumulated from zero in
            // loop order exactly like part0/part1/part2 of the reference
            if (lane == 0) sm.S[tri_idx(count, count)] = make_float4(0.f, 0.f, 0.f, 0.f);
            {
                float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
                float4 *row = sm.S + tri_idx(lane < 16 ? lane : 0, 0) + lane;  // &S(lane, lane)
                if (lane < count) row[0] = acc;
                if (LEAN) {
#pragma unroll 4
                    for (int s = 0; s < 16; ++s) {
                        if (s >= count) break;
                        if (lane + s < count) {
                            const float4 q = sm.PW[lane + s];
                            acc.x += q.x; acc.y += q.y; acc.z += q.z; acc.w += q.w;
                            row[s + 1] = acc;
                        }
                    }
                } else {
#pragma unroll
                    for (int s = 0; s < 16; ++s) {
                        if (s >= count) break;
                        if (lane + s < count) {
                            const float4 q = sm.PW[lane + s];
                            acc.x += q.x; acc.y += q.y; acc.z += q.z; acc.w += q.w;
                            row[s + 1] = acc;
                        }
                    }
                }
            }
            tm.sync();
            so.valid = it == 0;
            so.rank = my_rank;
            so.finite = finite;
        }
        xs = sm.S[count];  // S(0, count) == xsum_wsum

        // each lane's best starts at (run, 0): no entry is below 0, so a
        // candidate that only ties the running best never wins; NaN never
        // compares true
        LaneBest ob;
        ob.err = run;
        ob.ent = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) { ob.a[c] = 0.0f; ob.b[c] = 0.0f; }
        uint32_t lean_nq = 0;  // LEAN: candidates queued for the exact sweep below
        if (ncand <= 2u * TEAM || !prune) {
            if (LEAN) {
                uint32_t *queue = reinterpret_cast<uint32_t *>(sm.LB);
                for (uint32_t t = (uint32_t)lane; t < ncand; t += TEAM) queue[t] = t;
                lean_nq = ncand;
                tm.sync();
            } else {
                // short lists: the plain sweep, lane-strided over the candidates
                for (uint32_t t = (uint32_t)lane; t < ncand; t += TEAM) eval_candidate<NC>(sm, __ldg(tbl + t), xs, cw, ob);
            }
        } else {
            // 1. a lower bound of every candidate's error (see cand_bound)
            const BoundBlock bb = bound_block(xs, cw);
            float lmin = __int_as_float(0x7f800000);
            uint32_t tseed = 0xFFFFFFFFu;
            if (unit16) {
                const float4 *ub = (NC == 4 ? g_ub4 : g_ub3) + lane;
#pragma unroll (NITER > 1 ? 1 : 2)
                for (uint32_t t = (uint32_t)lane; t < ncand; t += TEAM, ub += TEAM) {
                    const float4 q = __ldg(ub);
                    const uint32_t o = __float_as_uint(q.w);
                    const float4 p0 = sm.S[o & 0xFFu];
                    const float4 p1 = sm.S[(o >> 8) & 0xFFu];
                    const float4 p2 = (NC == 4) ? sm.S[o >> 16] : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float bnd = unit_bound<NC>(p0, p1, p2, q, xs, cw, bb);
                    sm.LB[t] = bnd;
                    if (bnd < lmin) { lmin = bnd; tseed = t; }
                }
            } else {
#pragma unroll (NITER > 1 ? 1 : 2)
                for (uint32_t t = (uint32_t)lane; t < ncand; t += TEAM) {
                    const uint32_t e = __ldg(tbl + t);
                    const float4 p0 = sm.S[e & 0xFu];
                    const float4 p1 = sm.S[(e >> 4) & 0xFFu];
                    const float4 p2 = (NC == 4) ? sm.S[(e >> 12) & 0xFFu] : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float bnd = cand_bound<NC>(p0, p1, p2, lb_terms<NC>(p0.w, p1.w, p2.w, xs.w), cw, bb);
                    sm.LB[t] = bnd;
                    if (bnd < lmin) { lmin = bnd; tseed = t; }
                }
            }
            // 2. seeds: every lane's smallest bound, evaluated exactly; the
            // threshold is the smallest error reached (never above run)
            if (tseed != 0xFFFFFFFFu) {
                eval_candidate<NC>(sm, __ldg(tbl + tseed), xs, cw, ob);
                sm.LB[tseed] = __int_as_float(0x7f800000);  // already evaluated
            }
            const uint32_t ngroups = (ncand + 3u) >> 2;
            if (lane == 0) {
                for (uint32_t t = ncand; t < 4u * ngroups; ++t) sm.LB[t] = __int_as_float(0x7f800000);
                if (!unit16 && NITER == 1) {  // (the iterative kernels spill with it)
                    // one-cluster candidates: the flat bound of unit_terms with W =
                    // xs.w (their rounded alpha : beta : gamma are within a few u W of
                    // l^2 : (1-l)^2 : l(1-l), moving the error by at most 32 u W sum w
                    // on [0,1]^2, inside eps1; 2^-10 covers the approximate 1/W).  A
                    // seed among them may be written back to infinity, or evaluated
                    // again: either is harmless.
                    float rw;
                    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rw) : "f"(xs.w));
                    const float flat = __fmaf_rn(-(1.0f + 0x1p-10f) * bb.z, rw, -bb.eps1);
                    if (NC == 4) {
                        sm.LB[c_one4[count][0]] = flat;
                        sm.LB[c_one4[count][1]] = flat;
                    } else {
                        sm.LB[c_one3[count]] = flat;
                    }
                }
            }
            float thr = ob.err;
#pragma unroll
            for (int off = TEAM / 2; off > 0; off >>= 1) thr = fminf(thr, tm.shfl_xor(thr, off));
            tm.sync();
            // 3. survivors (bound not above thr; NaN = no bound) are packed in
            // place into the front of LB, four bounds per lane and round; a
            // round only writes slots that have already been read
            uint32_t *queue = reinterpret_cast<uint32_t *>(sm.LB);
            const float4 *lb4v = reinterpret_cast<const float4 *>(sm.LB);
            const unsigned below = (1u << lane) - 1u;
            uint32_t nq = 0;
            for (uint32_t r0 = 0; r0 < ngroups; r0 += TEAM) {
                const uint32_t g = r0 + (uint32_t)lane;
                float4 v = make_float4(__int_as_float(0x7f800000), __int_as_float(0x7f800000),
                                       __int_as_float(0x7f800000), __int_as_float(0x7f800000));
                if (g < ngroups) v = lb4v[g];
                const bool k0 = !(v.x > thr), k1 = !(v.y > thr), k2 = !(v.z > thr), k3 = !(v.w > thr);
                if (tm.ballot(k0 || k1 || k2 || k3) == 0u) continue;  // most rounds hold no survivor
                const unsigned b0 = tm.ballot(k0), b1 = tm.ballot(k1), b2 = tm.ballot(k2), b3 = tm.ballot(k3);
                const uint32_t n0 = (uint32_t)__popc(b0), n1 = (uint32_t)__popc(b1), n2 = (uint32_t)__popc(b2);
                if (k0) queue[nq + __popc(b0 & below)] = 4u * g;
                if (k1) queue[nq + n0 + __popc(b1 & below)] = 4u * g + 1u;
                if (k2) queue[nq + n0 + n1 + __popc(b2 & below)] = 4u * g + 2u;
                if (k3) queue[nq + n0 + n1 + n2 + __popc(b3 & below)] = 4u * g + 3u;
                nq += n0 + n1 + n2 + (uint32_t)__popc(b3);
            }
            tm.sync();
            // 4. exact errors of the survivors
            if (LEAN)
                lean_nq = nq;
            else
                for (uint32_t s = (uint32_t)lane; s < nq; s += TEAM) eval_candidate<NC>(sm, __ldg(tbl + queue[s]), xs, cw, ob);
        }
        if (LEAN) {
            const uint32_t *queue = reinterpret_cast<const uint32_t *>(sm.LB);
            for (uint32_t s = (uint32_t)lane; s < lean_nq; s += TEAM) eval_candidate<NC>(sm, __ldg(tbl + queue[s]), xs, cw, ob);
        }
        // lexicographic reduction of the lanes' bests; the winning lane (the
        // one holding the winning entry) supplies the endpoints
        float lbest = ob.err;
        uint32_t lent = ob.ent;
#pragma unroll
        for (int off = TEAM / 2; off > 0; off >>= 1) {
            const float oe = tm.shfl_xor(lbest, off);
            const uint32_t on = tm.shfl_xor(lent, off);
            if (oe < lbest || (oe == lbest && on < lent)) { lbest = oe; lent = on; }
        }
        if (lent != 0u) {
            const int src = __ffs(tm.ballot(ob.ent == lent)) - 1;
#pragma unroll
            for (int c = 0; c < 3; ++c) { ba[c] = tm.shfl(ob.a[c], src); bb[c] = tm.shfl(ob.b[c], src); }
            run = lbest;
            bentry = lent;
            bit = it;
            best_rank = my_rank;
            best_finite = finite;
        }
        tm.sync();  // the next ordering reuses the queue's shared memory
        if (bit != it) break;
        axis[0] = bb[0] - ba[0]; axis[1] = bb[1] - ba[1]; axis[2] = bb[2] - ba[2];
    }

    if (run < best_err) {
        int i, j, k;
        decode_entry(bentry, i, j, k);
        uint32_t ind = 3;
        // position of this pixel's point in the winning ordering: its rank, or
        // (with non-finite dot products) the last position < count holding it
        int maxpos = tm.shfl(best_rank, my_point >= 0 ? my_point : 0);
        if (!best_finite) {
            maxpos = -1;
            for (int m = 0; m < count; ++m) maxpos = (hist_get(sm, bit, m) == my_point) ? m : maxpos;
        }
        if (valid) {
            if (NC == 4) ind = maxpos >= k ? 1u : maxpos >= j ? 3u : maxpos >= i ? 2u : 0u;
            else ind = maxpos >= j ? 1u : maxpos >= i ? 2u : 0u;
        }
        const uint32_t word = __reduce_or_sync(tm.mask, lane < 16 ? (ind << (2 * lane)) : 0u);
        const uint32_t a565 = pack_565(ba[0], ba[1], ba[2]), b565 = pack_565(bb[0], bb[1], bb[2]);
        best = (NC == 4) ? write4(a565, b565, word) : write3(a565, b565, word);
        best_err = run;
    }
}

// Per-CTA inputs of the team path: the candidate lists for sets of fewer than
// 16 colours and the exact u8 -> [0,1] and sqrt(count) tables in shared memory.
struct TeamTables {
    const uint32_t *cand4, *cand3;
    const float *unorm, *sqrt;
};

template <int FMT, int TEAM, int NITER>
__device__ __forceinline__ uint2 colour_cluster_team(const Team<TEAM> &tm, TeamSmem &sm, const TeamTables &tt,
                                                     uint32_t px, bool inb, const DevParams &prm) {
    const uint32_t *tbl4 = tt.cand4, *tbl3 = tt.cand3;
    const int lane = tm.lane;
    const uint32_t a = px >> 24;
    const bool tr = (FMT == BC1) && inb && a < 128u;
    const bool valid = inb && !tr;
    const bool transparent = tm.ballot(tr) != 0u;
    const uint32_t key = valid ? (px & 0xFFFFFFu) : (0x01000000u | (uint32_t)lane);
    const unsigned eq = tm.match(key);
    const int first = __ffs(eq) - 1;
    const bool is_new = valid && first == lane;
    const unsigned newbits = tm.ballot(is_new);
    const int count = __popc(newbits);
    const int my_point = valid ? __popc(newbits & ((1u << first) - 1u)) : -1;

    // weights: count of equal pixels, or alpha weights summed in pixel order
    float wsum;
    if (!prm.alpha_weighted) {
        wsum = (float)__popc(eq);
    } else {
        const float wa = (float)(a + 1u) * (1.0f / 256.0f);
        const int fv = valid ? first : -1;
        wsum = 0.0f;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const float wq = tm.shfl(wa, q);
            const int fq = tm.shfl(fv, q);
            wsum = wsum + ((fq == lane) ? wq : 0.0f);
        }
    }
    if (is_new) {
        sm.P[0][my_point] = tt.unorm[px & 0xFFu];
        sm.P[1][my_point] = tt.unorm[(px >> 8) & 0xFFu];
        sm.P[2][my_point] = tt.unorm[(px >> 16) & 0xFFu];
        sm.P[3][my_point] = prm.alpha_weighted ? sqrt_rn(wsum) : tt.sqrt[__popc(eq)];
    }
    tm.sync();

    const uint32_t valid16 = tm.ballot(valid);
    if (count == 1) {
        int col[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) col[c] = f32_to_i32_clamped(sm.P[c][0] * 255.0f, 255);
        return single_fit<FMT>(col, valid16, transparent);
    }
    if (count == 0) {
        // RangeFit on an empty set (range.rs:67-98): start = end = 0, error 0.
        // BC1: compress3 writes (0, 0) with every pixel excluded -> index 3;
        // compress4 never wins against error 0.  BC2/3: write4 with a == b.
        return (FMT == BC1) ? make_uint2(0u, 0xFFFFFFFFu) : make_uint2(0u, 0u);
    }

    // Sym3x3::weighted_covariance (math.rs:44-73).  Lane k forms point k's
    // products; lane t then adds column t in point order, as the reference's
    // loop does.  Columns are padded with exact zeros to a multiple of 4
    // (x + 0 == x here: no running sum is -0, so no sign is lost).
    float *scr = sm.LB;  // free until the candidate sweep: [4][16] then [6][16]
    const int n4 = (count + 3) & ~3;
    float px3[3] = {0.f, 0.f, 0.f}, pw = 0.f;
    if (lane < count) { px3[0] = sm.P[0][lane]; px3[1] = sm.P[1][lane]; px3[2] = sm.P[2][lane]; pw = sm.P[3][lane]; }
    if (lane < 16) {
        scr[lane] = px3[0] * pw; scr[16 + lane] = px3[1] * pw; scr[32 + lane] = px3[2] * pw; scr[48 + lane] = pw;
    }
    tm.sync();
    const int col = lane < 10 ? lane : 0;
    auto column_sum = [&](const float *base) {
        float acc = 0.0f;
        for (int g = 0; g < n4; g += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(base + 16 * col + g);
            acc = acc + v.x; acc = acc + v.y; acc = acc + v.z; acc = acc + v.w;
        }
        return acc;
    };
    const float sum1 = column_sum(scr);  // lanes 0-2: centroid sums, lane 3: total
    const float total = tm.shfl(sum1, 3);
    const float cdiv = total > FLT_EPSILON ? div_rn(sum1, total) : sum1;
    const float cen[3] = {tm.shfl(cdiv, 0), tm.shfl(cdiv, 1), tm.shfl(cdiv, 2)};
    if (lane < 16) {
        const float a0 = px3[0] - cen[0], a1 = px3[1] - cen[1], a2 = px3[2] - cen[2];
        const float b0 = a0 * pw, b1 = a1 * pw, b2 = a2 * pw;
        const bool in = lane < count;
        float *c2 = scr + 64;
        c2[lane] = in ? a0 * b0 : 0.f;      c2[16 + lane] = in ? a0 * b1 : 0.f;
        c2[32 + lane] = in ? a0 * b2 : 0.f; c2[48 + lane] = in ? a1 * b1 : 0.f;
        c2[64 + lane] = in ? a1 * b2 : 0.f; c2[80 + lane] = in ? a2 * b2 : 0.f;
    }
    tm.sync();
    const float cv = column_sum(scr + 64);
    float cov[6];
#pragma unroll
    for (int t = 0; t < 6; ++t) cov[t] = tm.shfl(cv, t);
    tm.sync();  // the scratch is reused by the ordering
    float principal[3];
    principle_component_team(tm, cov, principal);

    const float cw[3] = {prm.w[0], prm.w[1], prm.w[2]};
    float best_err = FLT_MAX;
    uint2 best = make_uint2(0u, 0u);
    // 16 distinct colours without alpha weighting: every weight is sqrt(1) = 1
    const bool unit16 = count == 16 && !prm.alpha_weighted;
    if (count == 16) { tbl4 = g_cand16; tbl3 = g_cand16 + kCand4 + 1; }
    // the error bound used for pruning holds for finite, non-negative weights
    const bool prune = cw[0] >= 0.0f && cw[1] >= 0.0f && cw[2] >= 0.0f && cw[0] <= FLT_MAX && cw[1] <= FLT_MAX &&
                       cw[2] <= FLT_MAX;
    SharedOrder so{false, 0, false};
    if (FMT == BC1) {
        cluster_pass<3, TEAM, NITER, (NITER > 1)>(tm, sm, tbl3, count, principal, cw, prune, valid, my_point, unit16, best_err,
                                     best, so);
        if (!transparent)
            cluster_pass<4, TEAM, NITER, (NITER > 1)>(tm, sm, tbl4, count, principal, cw, prune, valid, my_point, unit16, best_err,
                                         best, so);
    } else {
        cluster_pass<4, TEAM, NITER>(tm, sm, tbl4, count, principal, cw, prune, valid, my_point, unit16, best_err,
                                     best, so);
    }
    return best;
}

template <int TEAM>
__device__ __forceinline__ uint2 team_bc3_alpha(const Team<TEAM> &tm, uint32_t v, bool inb) {
    const int lane = tm.lane;
    int min7 = (int)__reduce_min_sync(tm.mask, inb ? v : 255u);
    int max7 = (int)__reduce_max_sync(tm.mask, inb ? v : 0u);
    int min5 = (int)__reduce_min_sync(tm.mask, (inb && v != 0u) ? v : 255u);
    int max5 = (int)__reduce_max_sync(tm.mask, (inb && v != 255u) ? v : 0u);
    if (min5 > max5) min5 = max5;
    if (min7 > max7) min7 = max7;
    fix_range(min5, max5, 5);
    fix_range(min7, max7, 7);
    int c5[8], c7[8];
    c5[0] = min5; c5[1] = max5;
#pragma unroll
    for (int i = 1; i < 5; ++i) c5[1 + i] = ((5 - i) * min5 + i * max5) / 5;
    c5[6] = 0; c5[7] = 255;
    c7[0] = min5; c7[1] = max5;
#pragma unroll
    for (int i = 1; i < 7; ++i) c7[1 + i] = ((7 - i) * min7 + i * max7) / 7;
    int i5 = 0, i7 = 0, d5 = abs((int)v - c5[0]), d7 = abs((int)v - c7[0]);
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        const int e5 = abs((int)v - c5[j]), e7 = abs((int)v - c7[j]);
        if (e5 < d5) { d5 = e5; i5 = j; }
        if (e7 < d7) { d7 = e7; i7 = j; }
    }
    if (!inb) { i5 = 0; i7 = 0; d5 = 0; d7 = 0; }
    const uint32_t err5 = __reduce_add_sync(tm.mask, (uint32_t)(d5 * d5));
    const uint32_t err7 = __reduce_add_sync(tm.mask, (uint32_t)(d7 * d7));
    uint32_t a0, a1, idx;
    if (err5 <= err7) {
        a0 = (uint32_t)min5; a1 = (uint32_t)max5; idx = (uint32_t)i5;
        if (min5 > max5) {  // never true after fix_range (alpha.rs:146-165)
            a0 = (uint32_t)max5; a1 = (uint32_t)min5;
            idx = idx == 0 ? 1u : idx == 1 ? 0u : (idx <= 5 ? 7u - idx : idx);
        }
    } else {
        a0 = (uint32_t)min7; a1 = (uint32_t)max7; idx = (uint32_t)i7;
        if (min7 < max7) { a0 = (uint32_t)max7; a1 = (uint32_t)min7; idx = (9u - idx) & 7u; }
    }
    const uint32_t lo = __reduce_or_sync(tm.mask, (lane < 8) ? (idx << (3 * lane)) : 0u);
    const uint32_t hi = __reduce_or_sync(tm.mask, (lane >= 8 && lane < 16) ? (idx << (3 * (lane - 8))) : 0u);
    return make_uint2(a0 | (a1 << 8) | ((lo & 0xFFFFu) << 16), (lo >> 16) | (hi << 8));
}


// ===========================================================================
// block-level entry points

// Thread-per-block: encode and store block b (RangeFit / SingleColourFit path).
template <int FMT>
__device__ __forceinline__ void range_block(const SrcDesc &src, size_t b, const DevParams &prm, uint8_t *out,
                                            const float *s_unorm, const float *s_sqrt, const PointCol &pt) {
    uint32_t px[16];
    const uint32_t mask = load_block_rgba(src, b, px);
    // alpha first, so the alpha bytes are dead before the colour fit's registers peak
    uint2 al = make_uint2(0u, 0u);
    if (FMT == BC2) al = encode_bc2_alpha(px, mask);
    if (FMT == BC3) {
        uint32_t v[4];
        channel_words(px, 3, v);
        al = encode_bc3_alpha(v, mask);
    }
    const uint2 col = colour_range_thread<FMT>(px, mask, prm, s_unorm, s_sqrt, pt);
    if (FMT == BC1) reinterpret_cast<uint2 *>(out)[b] = col;
    else reinterpret_cast<uint4 *>(out)[b] = make_uint4(al.x, al.y, col.x, col.y);
}

// Pixel p of block b for lane p < 16 of a team (RGBA8, pixel order), and
// whether it lies inside the image / is selected by the block's mask.
struct TeamPixel {
    uint32_t px;
    bool inb;
};

__device__ __forceinline__ TeamPixel load_team_pixel(const SrcDesc &src, size_t b, int p) {
    TeamPixel r{0u, false};
    if (p < 16) {
        if (src.mode == 1) {
            r.px = __ldg(reinterpret_cast<const uint32_t *>(src.base + 64 * b) + p);
            r.inb = src.masks ? ((__ldg(src.masks + b) >> p) & 1u) : true;
        } else {
            uint32_t bx, by;
            block_coords(src, b, bx, by);
            const uint32_t x = 4 * bx + (p & 3), y = 4 * by + (p >> 2);
            r.inb = x < src.width && y < src.height;
            if (r.inb) r.px = ld_u32_any(src.base + (size_t)y * src.pitch + 4 * (size_t)x);
        }
    }
    return r;
}

// Team-per-block: encode and store block b (ClusterFit path) from its pixels.
template <int FMT, int TEAM, int NITER>
__device__ __forceinline__ void cluster_block_px(const Team<TEAM> &tm, TeamSmem &sm, const TeamTables &tt,
                                                 const TeamPixel tp, size_t b, const DevParams &prm, uint8_t *out) {
    const int p = tm.lane;
    const uint32_t px = tp.px;
    const bool inb = tp.inb;
    uint2 al = make_uint2(0u, 0u);
    if (FMT == BC2) {
        const uint32_t q = inb ? bc2_quant(px >> 24) : 0u;
        al.x = __reduce_or_sync(tm.mask, p < 8 ? q << (4 * p) : 0u);
        al.y = __reduce_or_sync(tm.mask, (p >= 8 && p < 16) ? q << (4 * (p - 8)) : 0u);
    } else if (FMT == BC3) {
        al = team_bc3_alpha<TEAM>(tm, px >> 24, inb);
    }
    const uint2 col = colour_cluster_team<FMT, TEAM, NITER>(tm, sm, tt, px, inb, prm);
    if (p == 0) {
        if (FMT == BC1) reinterpret_cast<uint2 *>(out)[b] = col;
        else reinterpret_cast<uint4 *>(out)[b] = make_uint4(al.x, al.y, col.x, col.y);
    }
    tm.sync();
}

// Team-per-block: load, encode and store block b.
template <int FMT, int TEAM, int NITER>
__device__ __forceinline__ void cluster_block(const Team<TEAM> &tm, TeamSmem &sm, const TeamTables &tt,
                                              const SrcDesc &src, size_t b, const DevParams &prm, uint8_t *out) {
    const int p = tm.lane;
    uint32_t px = 0;
    bool inb = false;
    if (p < 16) {
        if (src.mode == 1) {
            px = __ldg(reinterpret_cast<const uint32_t *>(src.base + 64 * b) + p);
            inb = src.masks ? ((__ldg(src.masks + b) >> p) & 1u) : true;
        } else {
            uint32_t bx, by;
            block_coords(src, b, bx, by);
            const uint32_t x = 4 * bx + (p & 3), y = 4 * by + (p >> 2);
            inb = x < src.width && y < src.height;
            if (inb) px = ld_u32_any(src.base + (size_t)y * src.pitch + 4 * (size_t)x);
        }
    }
    uint2 al = make_uint2(0u, 0u);
    if (FMT == BC2) {
        const uint32_t q = inb ? bc2_quant(px >> 24) : 0u;
        al.x = __reduce_or_sync(tm.mask, p < 8 ? q << (4 * p) : 0u);
        al.y = __reduce_or_sync(tm.mask, (p >= 8 && p < 16) ? q << (4 * (p - 8)) : 0u);
    } else if (FMT == BC3) {
        al = team_bc3_alpha<TEAM>(tm, px >> 24, inb);
    }
    const uint2 col = colour_cluster_team<FMT, TEAM, NITER>(tm, sm, tt, px, inb, prm);
    if (p == 0) {
        if (FMT == BC1) reinterpret_cast<uint2 *>(out)[b] = col;
        else reinterpret_cast<uint4 *>(out)[b] = make_uint4(al.x, al.y, col.x, col.y);
    }
    tm.sync();
}

// (F1, r, C, offsets) of unit_bound from exact weight-lane terms w = (alpha,
// beta, gamma, factor) of a weight-1, 16-point set (W = 16): A = alpha + beta +
// 2 gamma, B = alpha + gamma, f = 1/det.  det of the f32 values is exact in
// double (products of two 24-bit significands); each term is rounded once.
//
// det = 0 exactly when every point is in one cluster (one interpolation
// weight l; the f32 constants keep alpha : beta : gamma = l^2 : (1-l)^2 :
// l(1-l) exactly, as 4/9 and 2/9 are 4 and 2 times 1/9 in f32).  The fit is
// then a single colour c = l a + (1-l) b, whose error sum_c w_c (W c^2 -
// 2 X c) is at least -Z/W; the reference's rounded ax, bx move it by at most
// 4 u sum_c w_c X_c (a, b in [0,1]), inside eps1.  So such a candidate gets
// the flat bound -(1 + 2^-10) Z/W - eps1 (F1 = 0), which the fitted
// endpoints of a textured block beat, instead of no bound.
__device__ __forceinline__ float4 unit_terms(const float4 w, uint32_t offs, bool one_cluster) {
    const double al = w.x, be = w.y, ga = w.z;
    const double det = al * be - ga * ga;
    const double A = al + be + 2.0 * ga;
    const float nan = __int_as_float(0x7fc00000);  // no bound
    if (!(det > 0.0))
        return one_cluster ? make_float4(0.0f, 0.0f, (float)(-(1.0 + 0x1p-10) / 16.0), __uint_as_float(offs))
                           : make_float4(nan, 0.0f, nan, __uint_as_float(offs));
    return make_float4((float)(-A / det), (float)(2.0 * (al + ga) / A), (float)(-(al + 0x1p-13) / det),
                       __uint_as_float(offs));
}

// Fill the bound terms g_ub4 / g_ub3 from this TU's loop-order candidate
// lists: the w-lane sums of a 16-point, weight-1 set are S(a,b).w = b - a
// (exact small integers), and wterms4 / wterms3 are the reference's f32 code.
static __global__ void k_unit_terms() {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < kCand4) {
        int i, j, k;
        decode_entry(g_cand16[t], i, j, k);
        const uint32_t offs = (uint32_t)tri_idx(0, i) | (uint32_t)tri_idx(i, j) << 8 | (uint32_t)tri_idx(j, k) << 16;
        const bool one = (i == 16) + (j - i == 16) + (k - j == 16) + (16 - k == 16) == 1;
        g_ub4[t] = unit_terms(wterms4((float)i, (float)(j - i), (float)(k - j), 16.0f), offs, one);
    }
    if (t < kCand3) {
        int i, j, k;
        decode_entry(g_cand16[kCand4 + 1 + t], i, j, k);
        const uint32_t offs = (uint32_t)tri_idx(0, i) | (uint32_t)tri_idx(i, j) << 8;
        const bool one = (i == 16) + (j - i == 16) + (16 - j == 16) == 1;
        g_ub3[t] = unit_terms(wterms3((float)i, (float)(j - i), 16.0f), offs, one);
    }
}

// ===========================================================================
// host side: candidate lists + upload of this TU's tables

// Build the candidate lists and single-colour tables and copy them to the
// current device.
static inline cudaError_t upload_tables_this_tu(const uint32_t lut[4][256][2]) {
    // compress4: (i, j, k), 0 <= i < 16, i <= j <= 16, max(j,1) <= k <= 16
    struct C { int m, rank; uint32_t e; };
    C c4[kCand4], c3[kCand3];
    int n4 = 0, n3 = 0;
    for (int i = 0; i < 16; ++i)
        for (int j = i; j <= 16; ++j)
            for (int k = (j == 0 ? 1 : j); k <= 16; ++k) {
                const int m = (i + 1 > j ? i + 1 : j) > k ? (i + 1 > j ? i + 1 : j) : k;
                c4[n4].m = m;
                c4[n4].rank = n4;
                c4[n4].e = (uint32_t)i | ((uint32_t)tri_idx(i, j) << 4) | ((uint32_t)tri_idx(j, k) << 12) |
                           ((uint32_t)n4 << 20);
                ++n4;
            }
    for (int i = 0; i < 16; ++i)
        for (int j = (i == 0 ? 1 : i); j <= 16; ++j) {
            const int m = i + 1 > j ? i + 1 : j;
            c3[n3].m = m;
            c3[n3].rank = n3;
            c3[n3].e = (uint32_t)i | ((uint32_t)tri_idx(i, j) << 4) | ((uint32_t)n3 << 20);
            ++n3;
        }
    if (n4 != kCand4 || n3 != kCand3) return cudaErrorInvalidValue;
    uint32_t loop_tbl[kCand4 + 1 + kCand3 + 1] = {};
    for (int t = 0; t < kCand4; ++t) loop_tbl[t] = c4[t].e;
    for (int t = 0; t < kCand3; ++t) loop_tbl[kCand4 + 1 + t] = c3[t].e;
    auto sort_by_m = [](C *v, int n) {
        for (int a = 1; a < n; ++a) {  // stable insertion sort on m
            C t = v[a];
            int b = a;
            while (b > 0 && v[b - 1].m > t.m) { v[b] = v[b - 1]; --b; }
            v[b] = t;
        }
    };
    sort_by_m(c4, n4);
    sort_by_m(c3, n3);
    uint32_t tbl[kCand4 + 1 + kCand3 + 1] = {};
    uint32_t nc4[17] = {}, nc3[17] = {};
    for (int t = 0; t < kCand4; ++t) tbl[t] = c4[t].e;
    for (int t = 0; t < kCand3; ++t) tbl[kCand4 + 1 + t] = c3[t].e;
    for (int n = 0; n <= 16; ++n) {
        for (int t = 0; t < kCand4; ++t) nc4[n] += c4[t].m <= n ? 1u : 0u;
        for (int t = 0; t < kCand3; ++t) nc3[n] += c3[t].m <= n ? 1u : 0u;
    }
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(g_cand, tbl, sizeof(tbl))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(g_cand16, loop_tbl, sizeof(loop_tbl))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_ncand4, nc4, sizeof(nc4))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_ncand3, nc3, sizeof(nc3))) != cudaSuccess) return e;
    // positions of the one-cluster candidates in the list each count uses
    uint16_t one4[17][2] = {}, one3[17] = {};
    auto find = [](const uint32_t *list, int n, uint32_t key, uint32_t mask) {
        for (int t = 0; t < n; ++t)
            if ((list[t] & mask) == key) return (uint16_t)t;
        return (uint16_t)0;
    };
    for (int n = 1; n <= 16; ++n) {
        const uint32_t *l4 = n == 16 ? loop_tbl : tbl;
        const uint32_t *l3 = n == 16 ? loop_tbl + kCand4 + 1 : tbl + kCand4 + 1;
        const uint32_t m4 = 0xFFFFFu, m3 = 0xFFFu;  // the i, S(i,j), S(j,k) fields
        one4[n][0] = find(l4, kCand4, (uint32_t)tri_idx(0, 0) << 4 | (uint32_t)tri_idx(0, n) << 12, m4);
        one4[n][1] = find(l4, kCand4, (uint32_t)tri_idx(0, n) << 4 | (uint32_t)tri_idx(n, n) << 12, m4);
        one3[n] = find(l3, kCand3, (uint32_t)tri_idx(0, n) << 4, m3);
    }
    if ((e = cudaMemcpyToSymbol(c_one4, one4, sizeof(one4))) != cudaSuccess) return e;
    if ((e = cudaMemcpyToSymbol(c_one3, one3, sizeof(one3))) != cudaSuccess) return e;
    k_unit_terms<<<(kCand4 + 255) / 256, 256>>>();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_unorm_tables<<<1, 256>>>();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_lut, lut, sizeof(uint32_t) * 4 * 256 * 2);
}


}  // namespace tx
