/*
 * texpresso_oracle.c -- CPU oracle for the BCn block encoder.
 *
 * TEST INFRASTRUCTURE ONLY (see texpresso_oracle.h).  A plain-C restatement
 * of jansol/texpresso 2.0.2 lib/src/ that keeps every f32 operation of the
 * reference in the same order: no fused multiply-add, true IEEE division where
 * the reference divides, reciprocal-then-multiply where it multiplies by a
 * reciprocal, libm round/trunc/sqrt (all exactly specified).  Each function
 * cites the reference lines it follows.  Compile with
 *     -O3 -ffp-contract=off -fno-fast-math
 */
#include "texpresso_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------ */
/* Formats and sizes: lib/src/lib.rs:103-105, :159-179                       */

size_t txo_block_size(int format)
{
    return (format == TXO_BC1 || format == TXO_BC4) ? 8 : 16;
}

size_t txo_num_blocks(size_t size) { return (size + 3) / 4; }

size_t txo_compressed_size(int format, size_t width, size_t height)
{
    return txo_num_blocks(width) * txo_num_blocks(height) * txo_block_size(format);
}

/* ------------------------------------------------------------------------ */
/* Single-colour tables.  The reference stores them as data
 * (lib/src/colourfit/single_lut.rs:52-1086, inherited from libsquish).  They
 * are the output of libsquish's published generator: for every pair of
 * quantised endpoints (v1 outer, v2 inner) mark the 8-bit targets reached by
 * code 0 and by the first interpolant with error 0 (first pair wins), then
 * relax errors from the right and the left neighbour until stable.  The tests
 * check the result against SHA-256 digests of the reference tables. */

typedef struct { uint8_t start, end, error; } lut_src;
typedef struct { lut_src s[2]; } lut_row;

static lut_row g_lut[4][256]; /* 5_3, 6_3, 5_4, 6_4 */
static pthread_once_t g_lut_once = PTHREAD_ONCE_INIT;

static void lut_generate(lut_row *rows, int bits, int colours)
{
    int err[256][2], st[256][2], en[256][2];
    for (int t = 0; t < 256; ++t)
        for (int k = 0; k < 2; ++k) { err[t][k] = 255; st[t][k] = 0; en[t][k] = 0; }
    const int n = 1 << bits;
    for (int v1 = 0; v1 < n; ++v1) {
        for (int v2 = 0; v2 < n; ++v2) {
            int a = (v1 << (8 - bits)) | (v1 >> (2 * bits - 8));
            int b = (v2 << (8 - bits)) | (v2 >> (2 * bits - 8));
            int code[2];
            code[0] = a;
            code[1] = (colours == 3) ? (a + b) / 2 : (2 * a + b) / 3;
            for (int k = 0; k < 2; ++k) {
                int t = code[k];
                if (err[t][k] != 0) { st[t][k] = v1; en[t][k] = v2; err[t][k] = 0; }
            }
        }
    }
    for (;;) {
        int stable = 1;
        for (int k = 0; k < 2; ++k) {
            for (int t = 0; t < 256; ++t) {
                if (t != 255 && err[t][k] > err[t + 1][k] + 1) {
                    st[t][k] = st[t + 1][k]; en[t][k] = en[t + 1][k];
                    err[t][k] = err[t + 1][k] + 1; stable = 0;
                }
                if (t != 0 && err[t][k] > err[t - 1][k] + 1) {
                    st[t][k] = st[t - 1][k]; en[t][k] = en[t - 1][k];
                    err[t][k] = err[t - 1][k] + 1; stable = 0;
                }
            }
        }
        if (stable) break;
    }
    for (int t = 0; t < 256; ++t)
        for (int k = 0; k < 2; ++k) {
            rows[t].s[k].start = (uint8_t)st[t][k];
            rows[t].s[k].end = (uint8_t)en[t][k];
            rows[t].s[k].error = (uint8_t)err[t][k];
        }
}

static void lut_init(void)
{
    lut_generate(g_lut[0], 5, 3);
    lut_generate(g_lut[1], 6, 3);
    lut_generate(g_lut[2], 5, 4);
    lut_generate(g_lut[3], 6, 4);
}

void txo_single_lut(int which, uint8_t out[256 * 6])
{
    pthread_once(&g_lut_once, lut_init);
    for (int t = 0; t < 256; ++t)
        for (int k = 0; k < 2; ++k) {
            out[6 * t + 3 * k + 0] = g_lut[which][t].s[k].start;
            out[6 * t + 3 * k + 1] = g_lut[which][t].s[k].end;
            out[6 * t + 3 * k + 2] = g_lut[which][t].s[k].error;
        }
}

/* ------------------------------------------------------------------------ */
/* Math helpers: lib/src/math.rs:100-102, lib/src/math/vec3.rs:51-81        */

/* f32_to_i32_clamped: roundf(a).max(0).min(limit) as i32.  f32::max/min
 * return the non-NaN operand, as fmaxf/fminf do. */
static int f32_to_i32_clamped(float a, int limit)
{
    return (int)fminf(fmaxf(roundf(a), 0.0f), (float)limit);
}

static float dot3(const float a[3], const float b[3])
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* ------------------------------------------------------------------------ */
/* ColourSet: lib/src/colourset.rs:35-141                                   */

typedef struct {
    int count;
    float p[16][3];
    float w[16];
    int8_t remap[16];
    int transparent;
} colour_set;

static void colour_set_build(colour_set *s, const uint8_t *rgba, uint32_t mask, int format,
                             int alpha_weighted)
{
    memset(s, 0, sizeof(*s));
    for (int i = 0; i < 16; ++i) {
        const uint8_t *pi = rgba + 4 * i;
        if ((mask & (1u << i)) == 0) { s->remap[i] = -1; continue; }
        if (format == TXO_BC1 && pi[3] < 128) { s->remap[i] = -1; s->transparent = 1; continue; }
        for (int j = 0;; ++j) {
            if (j == i) {
                float x = (float)pi[0] / 255.0f;
                float y = (float)pi[1] / 255.0f;
                float z = (float)pi[2] / 255.0f;
                float w = (float)((int)pi[3] + 1) / 256.0f;
                s->p[s->count][0] = x;
                s->p[s->count][1] = y;
                s->p[s->count][2] = z;
                s->w[s->count] = alpha_weighted ? w : 1.0f;
                s->remap[i] = (int8_t)s->count;
                s->count += 1;
                break;
            }
            const uint8_t *pj = rgba + 4 * j;
            int dup = (mask & (1u << j)) != 0 && pi[0] == pj[0] && pi[1] == pj[1] &&
                      pi[2] == pj[2] && (format != TXO_BC1 || pj[3] >= 128);
            if (dup) {
                int idx = s->remap[j];
                float w = (float)((int)pi[3] + 1) / 256.0f;
                s->w[idx] += alpha_weighted ? w : 1.0f;
                s->remap[i] = (int8_t)idx;
                break;
            }
        }
    }
    for (int i = 0; i < 16; ++i) s->w[i] = sqrtf(s->w[i]);
}

static void remap_indices(const colour_set *s, const uint8_t source[16], uint8_t target[16])
{
    for (int i = 0; i < 16; ++i) {
        int j = s->remap[i];
        target[i] = (j == -1) ? 3 : source[j];
    }
}

/* ------------------------------------------------------------------------ */
/* Sym3x3: lib/src/math.rs:44-97                                            */

static void weighted_covariance(const colour_set *s, float cov[6])
{
    const int n = s->count;
    float total = 0.0f;
    for (int i = 0; i < n; ++i) total = total + s->w[i];
    float c[3] = {0.0f, 0.0f, 0.0f};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) c[k] = c[k] + s->p[i][k] * s->w[i];
    if (total > FLT_EPSILON)
        for (int k = 0; k < 3; ++k) c[k] = c[k] / total;
    for (int k = 0; k < 6; ++k) cov[k] = 0.0f;
    for (int i = 0; i < n; ++i) {
        float a[3], b[3];
        for (int k = 0; k < 3; ++k) a[k] = s->p[i][k] - c[k];
        for (int k = 0; k < 3; ++k) b[k] = a[k] * s->w[i];
        cov[0] += a[0] * b[0];
        cov[1] += a[0] * b[1];
        cov[2] += a[0] * b[2];
        cov[3] += a[1] * b[1];
        cov[4] += a[1] * b[2];
        cov[5] += a[2] * b[2];
    }
}

static void principle_component(const float m[6], float out[3])
{
    const float r0[4] = {m[0], m[1], m[2], 0.0f};
    const float r1[4] = {m[1], m[3], m[4], 0.0f};
    const float r2[4] = {m[2], m[4], m[5], 0.0f};
    float v[4] = {1.0f, 1.0f, 1.0f, 1.0f};
    for (int it = 0; it < 8; ++it) {
        float w[4];
        for (int l = 0; l < 4; ++l) w[l] = r0[l] * v[0];
        for (int l = 0; l < 4; ++l) w[l] = r1[l] * v[1] + w[l];
        for (int l = 0; l < 4; ++l) w[l] = r2[l] * v[2] + w[l];
        float a = fmaxf(w[0], fmaxf(w[1], w[2]));
        float ra = 1.0f / a;
        for (int l = 0; l < 4; ++l) v[l] = w[l] * ra;
    }
    out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
}

/* ------------------------------------------------------------------------ */
/* Colour block packing: lib/src/colourblock.rs:28-94                       */

static unsigned pack_565(const float c[3])
{
    unsigned r = (unsigned)f32_to_i32_clamped(31.0f * c[0], 31);
    unsigned g = (unsigned)f32_to_i32_clamped(63.0f * c[1], 63);
    unsigned b = (unsigned)f32_to_i32_clamped(31.0f * c[2], 31);
    return (r << 11) | (g << 5) | b;
}

static void write_block(unsigned a, unsigned b, const uint8_t idx[16], uint8_t *blk)
{
    blk[0] = (uint8_t)(a & 0xFF); blk[1] = (uint8_t)(a >> 8);
    blk[2] = (uint8_t)(b & 0xFF); blk[3] = (uint8_t)(b >> 8);
    for (int i = 0; i < 4; ++i)
        blk[4 + i] = (uint8_t)(((idx[4 * i + 3] & 3) << 6) | ((idx[4 * i + 2] & 3) << 4) |
                               ((idx[4 * i + 1] & 3) << 2) | (idx[4 * i] & 3));
}

static void write3(const float start[3], const float end[3], const uint8_t idx[16], uint8_t *blk)
{
    unsigned a = pack_565(start), b = pack_565(end);
    uint8_t r[16];
    memcpy(r, idx, 16);
    if (a > b) {
        unsigned t = a; a = b; b = t;
        for (int i = 0; i < 16; ++i) r[i] = (r[i] == 0) ? 1 : (r[i] == 1) ? 0 : r[i];
    }
    write_block(a, b, r, blk);
}

static void write4(const float start[3], const float end[3], const uint8_t idx[16], uint8_t *blk)
{
    unsigned a = pack_565(start), b = pack_565(end);
    uint8_t r[16];
    memset(r, 0, 16);
    if (a < b) {
        unsigned t = a; a = b; b = t;
        for (int i = 0; i < 16; ++i) r[i] = (uint8_t)((idx[i] ^ 1) & 3);
    } else if (a > b) {
        memcpy(r, idx, 16);
    }
    write_block(a, b, r, blk);
}

/* ------------------------------------------------------------------------ */
/* SingleColourFit: lib/src/colourfit/single.rs:58-164                      */

typedef struct {
    const colour_set *set;
    int format;
    float start[3], end[3];
    int index;
    unsigned error, best_error;
    uint8_t best[8];
} single_fit;

static void single_endpoints(single_fit *f, int t0, int t1, int t2)
{
    const lut_row *lut[3] = {g_lut[t0], g_lut[t1], g_lut[t2]};
    int colour[3];
    for (int c = 0; c < 3; ++c) colour[c] = f32_to_i32_clamped(f->set->p[0][c] * 255.0f, 255);
    f->error = 0xFFFFFFFFu;
    for (int index = 0; index < 2; ++index) {
        unsigned error = 0;
        const lut_src *src[3];
        for (int c = 0; c < 3; ++c) {
            src[c] = &lut[c][colour[c]].s[index];
            unsigned d = src[c]->error;
            error += d * d;
        }
        if (error < f->error) {
            f->start[0] = (float)src[0]->start / 31.0f;
            f->start[1] = (float)src[1]->start / 63.0f;
            f->start[2] = (float)src[2]->start / 31.0f;
            f->end[0] = (float)src[0]->end / 31.0f;
            f->end[1] = (float)src[1]->end / 63.0f;
            f->end[2] = (float)src[2]->end / 31.0f;
            f->index = 2 * index;
            f->error = error;
        }
    }
}

static void single_compress(const colour_set *set, int format, uint8_t out[8])
{
    single_fit f;
    memset(&f, 0, sizeof(f));
    f.set = set; f.format = format; f.error = f.best_error = 0xFFFFFFFFu;
    uint8_t src[16], idx[16];
    if (format == TXO_BC1) {
        single_endpoints(&f, 0, 1, 0); /* LOOKUP_5_3, 6_3, 5_3 */
        if (f.error < f.best_error) {
            memset(src, f.index, 16);
            remap_indices(set, src, idx);
            write3(f.start, f.end, idx, f.best);
            f.best_error = f.error;
        }
    }
    if (format != TXO_BC1 || !set->transparent) {
        single_endpoints(&f, 2, 3, 2); /* LOOKUP_5_4, 6_4, 5_4 */
        if (f.error < f.best_error) {
            memset(src, f.index, 16);
            remap_indices(set, src, idx);
            write4(f.start, f.end, idx, f.best);
            f.best_error = f.error;
        }
    }
    memcpy(out, f.best, 8);
}

/* ------------------------------------------------------------------------ */
/* RangeFit: lib/src/colourfit/range.rs:44-192                              */

typedef struct {
    const colour_set *set;
    float weights[3];
    float start[3], end[3];
    uint8_t indices[16];
    float best_error;
    uint8_t best[8];
} range_fit;

static void range_init(range_fit *f, const colour_set *set, const float weights[3])
{
    memset(f, 0, sizeof(*f));
    f->set = set;
    for (int k = 0; k < 3; ++k) f->weights[k] = weights[k];
    f->best_error = FLT_MAX;
    float cov[6], axis[3];
    weighted_covariance(set, cov);
    principle_component(cov, axis);
    float start[3] = {0, 0, 0}, end[3] = {0, 0, 0};
    if (set->count > 0) {
        memcpy(start, set->p[0], sizeof(start));
        memcpy(end, start, sizeof(end));
        float mn = dot3(start, axis), mx = mn;
        for (int i = 1; i < set->count; ++i) {
            float d = dot3(set->p[i], axis);
            if (d < mn) { memcpy(start, set->p[i], sizeof(start)); mn = d; }
            else if (d > mx) { memcpy(end, set->p[i], sizeof(end)); mx = d; }
        }
    }
    const float grid[3] = {31.0f, 63.0f, 31.0f};
    const float gridrcp[3] = {1.0f / 31.0f, 1.0f / 63.0f, 1.0f / 31.0f};
    for (int k = 0; k < 3; ++k) {
        float s = fminf(1.0f, fmaxf(0.0f, start[k]));
        float e = fminf(1.0f, fmaxf(0.0f, end[k]));
        f->start[k] = truncf(grid[k] * s + 0.5f) * gridrcp[k];
        f->end[k] = truncf(grid[k] * e + 0.5f) * gridrcp[k];
    }
}

static int range_helper(range_fit *f, const float (*codes)[3], int ncodes)
{
    const colour_set *s = f->set;
    uint8_t closest[16];
    memset(closest, 0, sizeof(closest));
    float error = 0.0f;
    for (int i = 0; i < s->count; ++i) {
        float dist = FLT_MAX;
        int idx = 0;
        for (int j = 0; j < ncodes; ++j) {
            float d[3];
            for (int k = 0; k < 3; ++k) d[k] = f->weights[k] * (s->p[i][k] - codes[j][k]);
            float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (dd < dist) { dist = dd; idx = j; }
        }
        closest[i] = (uint8_t)idx;
        error += dist;
    }
    if (error < f->best_error) {
        remap_indices(s, closest, f->indices);
        f->best_error = error;
        return 1;
    }
    return 0;
}

static void range_compress(const colour_set *set, int format, const float weights[3], uint8_t out[8])
{
    range_fit f;
    range_init(&f, set, weights);
    if (format == TXO_BC1) {
        float codes[3][3];
        for (int k = 0; k < 3; ++k) {
            codes[0][k] = f.start[k];
            codes[1][k] = f.end[k];
            codes[2][k] = f.start[k] * 0.5f + f.end[k] * 0.5f;
        }
        if (range_helper(&f, codes, 3)) write3(f.start, f.end, f.indices, f.best);
    }
    if (format != TXO_BC1 || !set->transparent) {
        float codes[4][3];
        for (int k = 0; k < 3; ++k) {
            codes[0][k] = f.start[k];
            codes[1][k] = f.end[k];
            codes[2][k] = f.start[k] * (2.0f / 3.0f) + f.end[k] * (1.0f / 3.0f);
            codes[3][k] = f.start[k] * (1.0f / 3.0f) + f.end[k] * (2.0f / 3.0f);
        }
        if (range_helper(&f, codes, 4)) write4(f.start, f.end, f.indices, f.best);
    }
    memcpy(out, f.best, 8);
}

/* ------------------------------------------------------------------------ */
/* ClusterFit: lib/src/colourfit/cluster.rs:33-417                          */

typedef struct {
    const colour_set *set;
    int format;
    float weights[4];
    int num_iterations;
    float principle[3];
    uint8_t order[8][16];
    float pw[16][4];
    float xsum[4];
    float best_error; /* every lane of the reference's best_error is equal */
    uint8_t best[8];
    txo_block_stats *stats;
} cluster_fit;

/* Stable ordering by f32 key with non-finite keys last (cluster.rs:89-100).
 * For 16 elements Rust's sort_unstable_by runs insertion sort, which keeps
 * equal keys in input order. */
static int dps_less(float a, float b)
{
    int fa = isfinite(a), fb = isfinite(b);
    if (!fa) return 0;
    if (!fb) return 1;
    return a < b;
}

static int construct_ordering(cluster_fit *f, const float axis[3], int iteration)
{
    const colour_set *s = f->set;
    const int count = s->count;
    int di[16];
    float dv[16];
    for (int i = 0; i < 16; ++i) { di[i] = 0; dv[i] = FLT_MAX; }
    for (int i = 0; i < count; ++i) { di[i] = i; dv[i] = dot3(s->p[i], axis); }
    for (int i = 1; i < 16; ++i) {
        int ti = di[i];
        float tv = dv[i];
        int j = i;
        while (j > 0 && dps_less(tv, dv[j - 1])) { di[j] = di[j - 1]; dv[j] = dv[j - 1]; --j; }
        di[j] = ti; dv[j] = tv;
    }
    for (int i = 0; i < 16; ++i) f->order[iteration][i] = (uint8_t)di[i];
    for (int it = 0; it < iteration; ++it)
        if (memcmp(f->order[iteration], f->order[it], 16) == 0) return 0;
    for (int k = 0; k < 4; ++k) f->xsum[k] = 0.0f;
    for (int i = 0; i < count; ++i) {
        int j = f->order[iteration][i];
        float p[4] = {s->p[j][0], s->p[j][1], s->p[j][2], 1.0f};
        for (int k = 0; k < 4; ++k) f->pw[i][k] = p[k] * s->w[j];
        for (int k = 0; k < 4; ++k) f->xsum[k] += f->pw[i][k];
    }
    return 1;
}

/* One least-squares candidate (cluster.rs:189-220 and :320-353).  alphax and
 * betax carry the w lane; the error only reads lanes x,y,z. */
static float cluster_candidate(const float alphax[4], const float betax[4], float ab,
                               const float weights[4], float a[3], float b[3])
{
    const float grid[3] = {31.0f, 63.0f, 31.0f};
    const float gridrcp[3] = {1.0f / 31.0f, 1.0f / 63.0f, 1.0f / 31.0f};
    const float alpha2 = alphax[3], beta2 = betax[3];
    const float factor = 1.0f / ((alpha2 * beta2) - ab * ab);
    for (int k = 0; k < 3; ++k) {
        float av = ((alphax[k] * beta2) - betax[k] * ab) * factor;
        float bv = ((betax[k] * alpha2) - alphax[k] * ab) * factor;
        av = fminf(1.0f, fmaxf(0.0f, av));
        bv = fminf(1.0f, fmaxf(0.0f, bv));
        a[k] = truncf(grid[k] * av + 0.5f) * gridrcp[k];
        b[k] = truncf(grid[k] * bv + 0.5f) * gridrcp[k];
    }
    float e5[3];
    for (int k = 0; k < 3; ++k) {
        float e1 = (a[k] * a[k]) * alpha2 + (b[k] * b[k] * beta2);
        float e2 = (a[k] * b[k] * ab) - a[k] * alphax[k];
        float e3 = e2 - b[k] * betax[k];
        float e4 = 2.0f * e3 + e1;
        e5[k] = e4 * weights[k];
    }
    return e5[0] + e5[1] + e5[2];
}

static void cluster_compress3(cluster_fit *f)
{
    const int count = f->set->count;
    const float hh[4] = {0.5f, 0.5f, 0.5f, 0.25f};
    float best_a[3] = {0, 0, 0}, best_b[3] = {0, 0, 0};
    float best_error = f->best_error;
    int best_iteration = 0, best_i = 0, best_j = 0;
    float axis[3] = {f->principle[0], f->principle[1], f->principle[2]};
    for (int iteration = 0; iteration < f->num_iterations; ++iteration) {
        if (!construct_ordering(f, axis, iteration)) break;
        if (f->stats) f->stats->iterations3 += 1;
        float part0[4] = {0, 0, 0, 0};
        for (int i = 0; i < count; ++i) {
            float part1[4] = {0, 0, 0, 0};
            if (i == 0) memcpy(part1, f->pw[0], sizeof(part1));
            int jmin = (i == 0) ? 1 : i;
            for (int j = jmin; j <= count; ++j) {
                float part2[4], alphax[4], betax[4], t[4], a[3], b[3];
                for (int k = 0; k < 4; ++k) part2[k] = f->xsum[k] - part1[k] - part0[k];
                for (int k = 0; k < 4; ++k) t[k] = part1[k] * hh[k];
                for (int k = 0; k < 4; ++k) alphax[k] = t[k] + part0[k];
                for (int k = 0; k < 4; ++k) betax[k] = t[k] + part2[k];
                float ab = t[3];
                float error = cluster_candidate(alphax, betax, ab, f->weights, a, b);
                if (f->stats) f->stats->candidates += 1;
                if (error < best_error) {
                    memcpy(best_a, a, sizeof(a)); memcpy(best_b, b, sizeof(b));
                    best_i = i; best_j = j; best_error = error; best_iteration = iteration;
                }
                if (j < count)
                    for (int k = 0; k < 4; ++k) part1[k] += f->pw[j][k];
            }
            for (int k = 0; k < 4; ++k) part0[k] += f->pw[i][k];
        }
        if (best_iteration != iteration) break;
        for (int k = 0; k < 3; ++k) axis[k] = best_b[k] - best_a[k];
    }
    if (best_error < f->best_error) {
        const uint8_t *order = f->order[best_iteration];
        uint8_t unordered[16], idx[16];
        memset(unordered, 0, 16);
        for (int m = best_i; m < best_j; ++m) unordered[order[m]] = 2;
        for (int m = best_j; m < count; ++m) unordered[order[m]] = 1;
        remap_indices(f->set, unordered, idx);
        write3(best_a, best_b, idx, f->best);
        f->best_error = best_error;
    }
}

static void cluster_compress4(cluster_fit *f)
{
    const int count = f->set->count;
    const float c13[4] = {1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 9.0f};
    const float c23[4] = {2.0f / 3.0f, 2.0f / 3.0f, 2.0f / 3.0f, 4.0f / 9.0f};
    const float twoninths = 2.0f / 9.0f;
    float best_a[3] = {0, 0, 0}, best_b[3] = {0, 0, 0};
    float best_error = f->best_error;
    int best_iteration = 0, best_i = 0, best_j = 0, best_k = 0;
    float axis[3] = {f->principle[0], f->principle[1], f->principle[2]};
    for (int iteration = 0; iteration < f->num_iterations; ++iteration) {
        if (!construct_ordering(f, axis, iteration)) break;
        if (f->stats) f->stats->iterations4 += 1;
        float part0[4] = {0, 0, 0, 0};
        for (int i = 0; i < count; ++i) {
            float part1[4] = {0, 0, 0, 0};
            for (int j = i; j <= count; ++j) {
                float part2[4] = {0, 0, 0, 0};
                if (j == 0) memcpy(part2, f->pw[0], sizeof(part2));
                int kmin = (j == 0) ? 1 : j;
                for (int kk = kmin; kk <= count; ++kk) {
                    float part3[4], alphax[4], betax[4], a[3], b[3];
                    for (int l = 0; l < 4; ++l) part3[l] = f->xsum[l] - part2[l] - part1[l] - part0[l];
                    for (int l = 0; l < 4; ++l)
                        alphax[l] = part2[l] * c13[l] + (part1[l] * c23[l] + part0[l]);
                    for (int l = 0; l < 4; ++l)
                        betax[l] = part1[l] * c13[l] + (part2[l] * c23[l] + part3[l]);
                    float ab = twoninths * (part1[3] + part2[3]);
                    float error = cluster_candidate(alphax, betax, ab, f->weights, a, b);
                    if (f->stats) f->stats->candidates += 1;
                    if (error < best_error) {
                        memcpy(best_a, a, sizeof(a)); memcpy(best_b, b, sizeof(b));
                        best_i = i; best_j = j; best_k = kk;
                        best_error = error; best_iteration = iteration;
                    }
                    if (kk < count)
                        for (int l = 0; l < 4; ++l) part2[l] += f->pw[kk][l];
                }
                if (j < count)
                    for (int l = 0; l < 4; ++l) part1[l] += f->pw[j][l];
            }
            for (int l = 0; l < 4; ++l) part0[l] += f->pw[i][l];
        }
        if (best_iteration != iteration) break;
        for (int k = 0; k < 3; ++k) axis[k] = best_b[k] - best_a[k];
    }
    if (best_error < f->best_error) {
        const uint8_t *order = f->order[best_iteration];
        uint8_t unordered[16], idx[16];
        memset(unordered, 0, 16);
        for (int m = best_i; m < best_j; ++m) unordered[order[m]] = 2;
        for (int m = best_j; m < count; ++m) unordered[order[m]] = 3;
        for (int m = best_k; m < count; ++m) unordered[order[m]] = 1;
        remap_indices(f->set, unordered, idx);
        write4(best_a, best_b, idx, f->best);
        f->best_error = best_error;
    }
}

static void cluster_compress(const colour_set *set, int format, const float weights[3],
                             int iterate, uint8_t out[8], txo_block_stats *stats)
{
    cluster_fit f;
    memset(&f, 0, sizeof(f));
    f.set = set;
    f.format = format;
    f.weights[0] = weights[0]; f.weights[1] = weights[1]; f.weights[2] = weights[2];
    f.weights[3] = 1.0f;
    f.num_iterations = iterate ? 8 : 1;
    f.best_error = FLT_MAX;
    f.stats = stats;
    float cov[6];
    weighted_covariance(set, cov);
    principle_component(cov, f.principle);
    /* ColourFit::compress, lib/src/colourfit.rs:44-60 */
    if (format == TXO_BC1) {
        cluster_compress3(&f);
        if (!set->transparent) cluster_compress4(&f);
    } else {
        cluster_compress4(&f);
    }
    memcpy(out, f.best, 8);
}

/* ------------------------------------------------------------------------ */
/* Alpha: lib/src/alpha.rs:27-256                                           */

static void compress_bc2(const uint8_t *rgba, uint32_t mask, uint8_t out[8])
{
    for (int i = 0; i < 8; ++i) {
        float a1 = (float)rgba[4 * (2 * i) + 3] * (15.0f / 255.0f);
        float a2 = (float)rgba[4 * (2 * i + 1) + 3] * (15.0f / 255.0f);
        int q1 = f32_to_i32_clamped(a1, 15);
        int q2 = f32_to_i32_clamped(a2, 15);
        if ((mask & (1u << (2 * i))) == 0) q1 = 0;
        if ((mask & (1u << (2 * i + 1))) == 0) q2 = 0;
        out[i] = (uint8_t)(q1 | (q2 << 4));
    }
}

static void fix_range(int *mn, int *mx, int steps)
{
    if (*mx - *mn < steps) *mx = (*mn + steps < 255) ? *mn + steps : 255;
    if (*mx - *mn < steps) *mn = (*mx - steps > 0) ? *mx - steps : 0;
}

static unsigned fit_codes(const uint8_t *rgba, int channel, uint32_t mask, const int codes[8],
                          uint8_t idx[16])
{
    unsigned err = 0;
    for (int i = 0; i < 16; ++i) {
        if ((mask & (1u << i)) == 0) { idx[i] = 0; continue; }
        int v = rgba[4 * i + channel];
        unsigned least = 0xFFFFFFFFu;
        int index = 0;
        for (int j = 0; j < 8; ++j) {
            int d = v - codes[j];
            unsigned dd = (unsigned)(d * d);
            if (dd < least) { least = dd; index = j; }
        }
        idx[i] = (uint8_t)index;
        err += least;
    }
    return err;
}

static void write_alpha_block(int a0, int a1, const uint8_t idx[16], uint8_t out[8])
{
    out[0] = (uint8_t)a0;
    out[1] = (uint8_t)a1;
    for (int i = 0; i < 2; ++i) {
        uint32_t v = 0;
        for (int j = 0; j < 8; ++j) v |= (uint32_t)idx[8 * i + j] << (3 * j);
        for (int j = 0; j < 3; ++j) out[2 + 3 * i + j] = (uint8_t)((v >> (8 * j)) & 0xFF);
    }
}

static void compress_bc3(const uint8_t *rgba, int channel, uint32_t mask, uint8_t out[8],
                         int *mode)
{
    int min5 = 255, max5 = 0, min7 = 255, max7 = 0;
    for (int i = 0; i < 16; ++i) {
        if ((mask & (1u << i)) == 0) continue;
        int v = rgba[4 * i + channel];
        if (v < min7) min7 = v;
        if (v > max7) max7 = v;
        if (v != 0 && v < min5) min5 = v;
        if (v != 255 && v > max5) max5 = v;
    }
    if (min5 > max5) min5 = max5;
    if (min7 > max7) min7 = max7;
    fix_range(&min5, &max5, 5);
    fix_range(&min7, &max7, 7);
    int codes5[8], codes7[8];
    codes5[0] = min5; codes5[1] = max5;
    for (int i = 1; i < 5; ++i) codes5[1 + i] = ((5 - i) * min5 + i * max5) / 5;
    codes5[6] = 0; codes5[7] = 255;
    /* codes7[0..2] are min5/max5, as in alpha.rs:237-239 */
    codes7[0] = min5; codes7[1] = max5;
    for (int i = 1; i < 7; ++i) codes7[1 + i] = ((7 - i) * min7 + i * max7) / 7;
    uint8_t i5[16], i7[16];
    unsigned e5 = fit_codes(rgba, channel, mask, codes5, i5);
    unsigned e7 = fit_codes(rgba, channel, mask, codes7, i7);
    if (e5 <= e7) {
        /* write_alpha_block5 (alpha.rs:146-165) */
        if (min5 > max5) {
            uint8_t sw[16];
            for (int i = 0; i < 16; ++i) {
                int x = i5[i];
                sw[i] = (uint8_t)(x == 0 ? 1 : x == 1 ? 0 : (x >= 2 && x <= 5) ? 7 - x : x);
            }
            write_alpha_block(max5, min5, sw, out);
        } else {
            write_alpha_block(min5, max5, i5, out);
        }
        if (mode) *mode = 5;
    } else {
        /* write_alpha_block7 (alpha.rs:167-185) */
        if (min7 < max7) {
            uint8_t sw[16];
            for (int i = 0; i < 16; ++i) {
                int x = i7[i];
                sw[i] = (uint8_t)(x == 0 ? 1 : x == 1 ? 0 : 9 - x);
            }
            write_alpha_block(max7, min7, sw, out);
        } else {
            write_alpha_block(min7, max7, i7, out);
        }
        if (mode) *mode = 7;
    }
}

/* ------------------------------------------------------------------------ */
/* Format::compress_block_masked: lib/src/lib.rs:188-234                    */

void txo_compress_block_masked(int format, const uint8_t rgba[64], uint32_t mask,
                               const txo_params *params, uint8_t *out, txo_block_stats *stats)
{
    pthread_once(&g_lut_once, lut_init);
    if (stats) memset(stats, 0, sizeof(*stats));
    int *m0 = stats ? &stats->alpha_mode[0] : NULL;
    int *m1 = stats ? &stats->alpha_mode[1] : NULL;
    switch (format) {
    case TXO_BC2: compress_bc2(rgba, mask, out); break;
    case TXO_BC3: compress_bc3(rgba, 3, mask, out, m0); break;
    case TXO_BC4: compress_bc3(rgba, 0, mask, out, m0); break;
    case TXO_BC5:
        compress_bc3(rgba, 0, mask, out, m0);
        compress_bc3(rgba, 1, mask, out + 8, m1);
        break;
    default: break;
    }
    if (format == TXO_BC1 || format == TXO_BC2 || format == TXO_BC3) {
        colour_set set;
        colour_set_build(&set, rgba, mask, format, params->weigh_colour_by_alpha != 0);
        uint8_t *colour = out + (format == TXO_BC1 ? 0 : 8);
        if (stats) stats->count = set.count;
        if (set.count == 1) {
            if (stats) stats->path = 1;
            single_compress(&set, format, colour);
        } else if (params->algorithm == TXO_RANGE_FIT || set.count == 0) {
            if (stats) stats->path = 2;
            range_compress(&set, format, params->weights, colour);
        } else {
            if (stats) stats->path = 3;
            cluster_compress(&set, format, params->weights,
                             params->algorithm == TXO_ITERATIVE_CLUSTER_FIT, colour, stats);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Format::compress: lib/src/lib.rs:287-335, block rows over threads         */

typedef struct {
    int format;
    const uint8_t *rgba;
    size_t width, height, bw, nrows, nblocks_total;
    const txo_params *params;
    uint8_t *out;
    atomic_size_t next_row;
} compress_job;

static void compress_row(compress_job *job, size_t y)
{
    const size_t bs = txo_block_size(job->format);
    uint8_t src[64];
    memset(src, 0, sizeof(src));
    for (size_t x = 0; x < job->bw; ++x) {
        size_t b = y * job->bw + x;
        if (b >= job->nblocks_total) break;
        uint32_t mask = 0;
        for (int py = 0; py < 4; ++py)
            for (int px = 0; px < 4; ++px) {
                size_t sx = 4 * x + (size_t)px, sy = 4 * y + (size_t)py;
                int index = 4 * py + px;
                if (sx < job->width && sy < job->height) {
                    memcpy(src + 4 * index, job->rgba + 4 * (job->width * sy + sx), 4);
                    mask |= 1u << index;
                }
            }
        txo_compress_block_masked(job->format, src, mask, job->params, job->out + b * bs, NULL);
    }
}

static void *compress_worker(void *arg)
{
    compress_job *job = (compress_job *)arg;
    for (;;) {
        size_t y = atomic_fetch_add(&job->next_row, 1);
        if (y >= job->nrows) break;
        compress_row(job, y);
    }
    return NULL;
}

int txo_online_cores(void)
{
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

static void run_workers(void *(*fn)(void *), void *job, int nthreads)
{
    if (nthreads <= 0) nthreads = txo_online_cores();
    if (nthreads == 1) { fn(job); return; }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    int started = 0;
    for (int t = 0; t < nthreads; ++t)
        if (pthread_create(&th[t], NULL, fn, job) == 0) ++started;
    if (started == 0) fn(job);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
}

int txo_compress(int format, const uint8_t *rgba, size_t width, size_t height,
                 const txo_params *params, uint8_t *out, size_t out_len, int nthreads)
{
    pthread_once(&g_lut_once, lut_init);
    if (out_len < txo_compressed_size(format, width, height)) return -1;
    if (width == 0) return -1; /* chunk size 0 panics in the reference */
    const size_t bs = txo_block_size(format);
    if (out_len % bs != 0) return -1; /* a trailing partial block panics */
    compress_job job;
    job.format = format;
    job.rgba = rgba;
    job.width = width;
    job.height = height;
    job.bw = txo_num_blocks(width);
    /* every full block of the output is written: rows past the image get
     * fully masked blocks (lib.rs:300-305 chunks the whole output) */
    job.nblocks_total = out_len / bs;
    job.nrows = (job.nblocks_total + job.bw - 1) / job.bw;
    job.params = params;
    job.out = out;
    atomic_init(&job.next_row, 0);
    run_workers(compress_worker, &job, nthreads);
    return 0;
}

typedef struct {
    int format;
    const uint8_t *blocks;
    const uint32_t *masks;
    size_t n;
    const txo_params *params;
    uint8_t *out;
    txo_block_stats *stats;
    atomic_size_t next;
} blocks_job;

static void *blocks_worker(void *arg)
{
    blocks_job *job = (blocks_job *)arg;
    const size_t bs = txo_block_size(job->format);
    const size_t chunk = 64;
    for (;;) {
        size_t b0 = atomic_fetch_add(&job->next, chunk);
        if (b0 >= job->n) break;
        size_t b1 = b0 + chunk < job->n ? b0 + chunk : job->n;
        for (size_t b = b0; b < b1; ++b)
            txo_compress_block_masked(job->format, job->blocks + 64 * b,
                                      job->masks ? job->masks[b] : 0xFFFFu, job->params,
                                      job->out + b * bs, job->stats ? &job->stats[b] : NULL);
    }
    return NULL;
}

void txo_compress_blocks(int format, const uint8_t *blocks, const uint32_t *masks,
                         size_t nblocks, const txo_params *params, uint8_t *out,
                         txo_block_stats *stats, int nthreads)
{
    pthread_once(&g_lut_once, lut_init);
    blocks_job job;
    job.format = format;
    job.blocks = blocks;
    job.masks = masks;
    job.n = nblocks;
    job.params = params;
    job.out = out;
    job.stats = stats;
    atomic_init(&job.next, 0);
    run_workers(blocks_worker, &job, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Decoders: lib/src/colourblock.rs:97-169, lib/src/alpha.rs:53-68,258-304,
 * lib/src/lib.rs:124-156,240-277                                           */

static void unpack_565(unsigned v, uint8_t c[4])
{
    unsigned r = (v >> 11) & 0x1F, g = (v >> 5) & 0x3F, b = v & 0x1F;
    c[0] = (uint8_t)((r << 3) | (r >> 2));
    c[1] = (uint8_t)((g << 2) | (g >> 4));
    c[2] = (uint8_t)((b << 3) | (b >> 2));
    c[3] = 255;
}

static void decompress_colour(const uint8_t *blk, int is_bc1, uint8_t rgba[64])
{
    uint8_t codes[16];
    unsigned a = (unsigned)blk[0] | ((unsigned)blk[1] << 8);
    unsigned b = (unsigned)blk[2] | ((unsigned)blk[3] << 8);
    unpack_565(a, codes);
    unpack_565(b, codes + 4);
    for (int i = 0; i < 4; ++i) {
        unsigned c = codes[i], d = codes[4 + i];
        if (is_bc1 && a <= b) {
            codes[8 + i] = (uint8_t)((c + d) / 2);
            codes[12 + i] = 0;
        } else {
            codes[8 + i] = (uint8_t)((2 * c + d) / 3);
            codes[12 + i] = (uint8_t)((c + 2 * d) / 3);
        }
    }
    codes[8 + 3] = 255;
    codes[12 + 3] = (is_bc1 && a <= b) ? 0 : 255;
    for (int i = 0; i < 16; ++i) {
        int idx = (blk[4 + i / 4] >> (2 * (i % 4))) & 3;
        memcpy(rgba + 4 * i, codes + 4 * idx, 4);
    }
}

static void decompress_bc2(uint8_t rgba[64], const uint8_t *blk)
{
    for (int i = 0; i < 8; ++i) {
        uint8_t q = blk[i], lo = q & 0x0F, hi = q & 0xF0;
        rgba[4 * (2 * i) + 3] = (uint8_t)(lo | (lo << 4));
        rgba[4 * (2 * i + 1) + 3] = (uint8_t)(hi | (hi >> 4));
    }
}

static void decompress_bc3(uint8_t rgba[64], int channel, const uint8_t *blk)
{
    int a0 = blk[0], a1 = blk[1];
    int codes[8];
    codes[0] = a0; codes[1] = a1;
    if (a0 <= a1) {
        for (int i = 1; i < 5; ++i) codes[1 + i] = ((5 - i) * a0 + i * a1) / 5;
        codes[6] = 0; codes[7] = 255;
    } else {
        for (int i = 1; i < 7; ++i) codes[1 + i] = ((7 - i) * a0 + i * a1) / 7;
    }
    for (int h = 0; h < 2; ++h) {
        uint32_t v = (uint32_t)blk[2 + 3 * h] | ((uint32_t)blk[3 + 3 * h] << 8) |
                     ((uint32_t)blk[4 + 3 * h] << 16);
        for (int j = 0; j < 8; ++j) rgba[4 * (8 * h + j) + channel] = (uint8_t)codes[(v >> (3 * j)) & 7];
    }
}

void txo_decompress_block(int format, const uint8_t *block, uint8_t rgba[64])
{
    if (format == TXO_BC1 || format == TXO_BC2 || format == TXO_BC3) {
        decompress_colour(block + (format == TXO_BC1 ? 0 : 8), format == TXO_BC1, rgba);
    } else {
        for (int i = 0; i < 16; ++i) {
            rgba[4 * i + 0] = 0; rgba[4 * i + 1] = 0; rgba[4 * i + 2] = 0; rgba[4 * i + 3] = 255;
        }
    }
    switch (format) {
    case TXO_BC2: decompress_bc2(rgba, block); break;
    case TXO_BC3: decompress_bc3(rgba, 3, block); break;
    case TXO_BC4:
        decompress_bc3(rgba, 0, block);
        for (int i = 0; i < 16; ++i) { rgba[4 * i + 1] = rgba[4 * i]; rgba[4 * i + 2] = rgba[4 * i]; }
        break;
    case TXO_BC5:
        decompress_bc3(rgba, 0, block);
        decompress_bc3(rgba, 1, block + 8);
        break;
    default: break;
    }
}

int txo_decompress(int format, const uint8_t *data, size_t data_len, size_t width,
                   size_t height, uint8_t *out, size_t out_len)
{
    const size_t bw = txo_num_blocks(width), bs = txo_block_size(format);
    if (width == 0) return -1;
    const size_t row_bytes = width * 16;
    const size_t nrows = (out_len + row_bytes - 1) / row_bytes;
    for (size_t y = 0; y < nrows; ++y) {
        for (size_t x = 0; x < bw; ++x) {
            size_t off = (x + y * bw) * bs;
            if (off + bs > data_len) return -1;
            uint8_t rgba[64];
            txo_decompress_block(format, data + off, rgba);
            for (int py = 0; py < 4; ++py)
                for (int px = 0; px < 4; ++px) {
                    size_t sx = 4 * x + (size_t)px, sy = (size_t)py;
                    if (sx < width && 4 * y + sy < height) {
                        size_t o = y * row_bytes + 4 * (sx + sy * width);
                        if (o + 4 <= out_len) memcpy(out + o, rgba + 4 * (px + 4 * py), 4);
                    }
                }
        }
    }
    return 0;
}
