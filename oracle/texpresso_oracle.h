/*
 * texpresso_oracle.h -- CPU oracle for the BCn block encoder.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Rust crate's block path (jansol/texpresso 2.0.2, lib/src/), written to
 * reproduce its f32 operation order exactly.  It exists to check the CUDA
 * library and to time the reference's CPU algorithm; no product code path may
 * link or call it.  Build flags must keep IEEE f32 semantics:
 * -O3 -ffp-contract=off -fno-fast-math (GCC contracts a*b+c into FMA on
 * aarch64 unless told not to; the reference never fuses).
 *
 * Parity pins: the eight known-answer blocks of lib/src/test_data.rs:15-135
 * (under all three algorithms, lib/src/lib.rs:369-393), the decoder cases of
 * lib/src/lib.rs:363-367,416-444, and the SHA-256 of the four single-colour
 * tables of lib/src/colourfit/single_lut.rs (regenerated here, not copied).
 */
#ifndef TEXPRESSO_ORACLE_H
#define TEXPRESSO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* lib/src/lib.rs:39-46 */
enum { TXO_BC1 = 0, TXO_BC2 = 1, TXO_BC3 = 2, TXO_BC4 = 3, TXO_BC5 = 4 };
/* lib/src/lib.rs:49-59 */
enum { TXO_RANGE_FIT = 0, TXO_CLUSTER_FIT = 1, TXO_ITERATIVE_CLUSTER_FIT = 2 };

/* lib/src/lib.rs:76-90 */
typedef struct txo_params {
    int32_t algorithm;
    float weights[3];
    int32_t weigh_colour_by_alpha;
} txo_params;

/* Per-block trace of what the encoder did (for tests and work accounting). */
typedef struct txo_block_stats {
    int32_t count;          /* distinct colours in the ColourSet           */
    int32_t path;           /* 0 none, 1 single, 2 range, 3 cluster         */
    int32_t iterations3;    /* cluster sweeps run by compress3              */
    int32_t iterations4;    /* cluster sweeps run by compress4              */
    int64_t candidates;     /* cluster candidate evaluations                */
    int32_t alpha_mode[2];  /* per alpha channel: 5 or 7 codebook, 0 none   */
} txo_block_stats;

size_t txo_block_size(int format);
size_t txo_num_blocks(size_t size);
size_t txo_compressed_size(int format, size_t width, size_t height);

/* The four single-colour tables (256 rows x 6 bytes) in the order
 * 5_3, 6_3, 5_4, 6_4, regenerated from their published construction. */
void txo_single_lut(int which, uint8_t out[256 * 6]);

/* lib/src/lib.rs:188-234.  out must hold block_size(format) bytes. */
void txo_compress_block_masked(int format, const uint8_t rgba[64], uint32_t mask,
                               const txo_params *params, uint8_t *out,
                               txo_block_stats *stats /* may be NULL */);

/* lib/src/lib.rs:287-335.  Returns 0, or -1 when out_len is too small or the
 * width is zero (the reference panics there).  Blocks are spread over
 * nthreads pthreads one block row at a time, as rayon does (nthreads <= 0
 * means all online cores). */
int txo_compress(int format, const uint8_t *rgba, size_t width, size_t height,
                 const txo_params *params, uint8_t *out, size_t out_len, int nthreads);

/* Compress an explicit list of blocks (64 B RGBA + mask each).  Used for the
 * bounded CPU-baseline sample and for per-block statistics. */
void txo_compress_blocks(int format, const uint8_t *blocks, const uint32_t *masks,
                         size_t nblocks, const txo_params *params, uint8_t *out,
                         txo_block_stats *stats /* may be NULL */, int nthreads);

/* lib/src/lib.rs:240-277 and :124-156. */
void txo_decompress_block(int format, const uint8_t *block, uint8_t rgba[64]);
int txo_decompress(int format, const uint8_t *data, size_t data_len, size_t width,
                   size_t height, uint8_t *out, size_t out_len);

int txo_online_cores(void);

#ifdef __cplusplus
}
#endif
#endif
