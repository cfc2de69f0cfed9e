/*
 * texpresso_gb300.h -- C ABI of the GB300 (sm_103a) BCn block encoder.
 *
 * This is the drop-in boundary for jansol/texpresso's block-compression path.
 * Every entry point cites the reference interface it replaces
 * (paths relative to the texpresso repository).  Conventions:
 *   - plain pointers and sizes, no C++ or framework types;
 *   - every function returns TX_OK (0) or a negative TX_ERR_* status and
 *     never aborts the process (the reference panics where these return an
 *     error; a Rust veneer maps a negative status back to that panic);
 *   - host-buffer entry points are synchronous and thread-safe;
 *   - *_device entry points take device pointers and a cudaStream_t (passed
 *     as void*), are stream-ordered and return after enqueueing work.
 * There is no CPU fallback: without a usable CUDA device the compute entry
 * points return TX_ERR_NO_DEVICE.
 */
#ifndef TEXPRESSO_GB300_H
#define TEXPRESSO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TX_API __attribute__((visibility("default")))
#else
#define TX_API
#endif

/* Format -- lib/src/lib.rs:39-46 (enum Format { Bc1, Bc2, Bc3, Bc4, Bc5 }) */
#define TX_FORMAT_BC1 0
#define TX_FORMAT_BC2 1
#define TX_FORMAT_BC3 2
#define TX_FORMAT_BC4 3
#define TX_FORMAT_BC5 4

/* Algorithm -- lib/src/lib.rs:49-59 */
#define TX_RANGE_FIT 0
#define TX_CLUSTER_FIT 1
#define TX_ITERATIVE_CLUSTER_FIT 2

/* Status codes (the reference has none: it panics, lib/src/lib.rs:295). */
#define TX_OK 0
#define TX_ERR_INVALID_FORMAT (-1)
#define TX_ERR_INVALID_ARGUMENT (-2)
#define TX_ERR_OUTPUT_TOO_SMALL (-3)
#define TX_ERR_INPUT_TOO_SMALL (-4)
#define TX_ERR_CUDA (-5)
#define TX_ERR_NO_DEVICE (-6)
#define TX_ERR_TIMEOUT (-7)
#define TX_ERR_OUT_OF_MEMORY (-8)
#define TX_ERR_MISALIGNED (-9)
#define TX_ERR_BUSY (-10)
#define TX_ERR_CANCELLED (-11)

/* Params -- lib/src/lib.rs:76-90.  weigh_colour_by_alpha is 0 or 1. */
typedef struct tx_params {
    int32_t algorithm;
    float weights[3];
    int32_t weigh_colour_by_alpha;
} tx_params;

/* Params::default -- lib/src/lib.rs:92-100 (ClusterFit, perceptual
 * weights [0.2126, 0.7152, 0.0722] from lib/src/lib.rs:74, no alpha
 * weighting). */
TX_API void tx_params_default(tx_params *params);

/* Human-readable text for a status code (static storage). */
TX_API const char *tx_status_string(int status);

/* num_blocks -- lib/src/lib.rs:103-105 */
TX_API size_t tx_num_blocks(size_t size);

/* Format::block_size -- lib/src/lib.rs:159-168.  0 for an unknown format. */
TX_API size_t tx_block_size(int format);

/* Format::compressed_size -- lib/src/lib.rs:175-179.  0 for an unknown format. */
TX_API size_t tx_compressed_size(int format, size_t width, size_t height);

/* Format::compress -- lib/src/lib.rs:287-335.
 * rgba: tightly packed RGBA8, 4*width*height bytes (rgba_len >= that).
 * output: output_len >= tx_compressed_size(format, width, height).  As in
 * the reference every full block of output is written: rows below the image
 * receive fully masked blocks.  A width of 0, or an output_len that leaves a
 * partial trailing block, returns TX_ERR_INVALID_ARGUMENT (both panic in the
 * reference).  Host buffers; synchronous. */
TX_API int tx_compress(int format, const uint8_t *rgba, size_t rgba_len, size_t width,
                       size_t height, const tx_params *params, uint8_t *output,
                       size_t output_len);

/* Format::compress_block_masked -- lib/src/lib.rs:188-234.
 * rgba: 16 pixels (64 bytes), mask bit 4*y+x marks a valid pixel.
 * output_len >= tx_block_size(format).  Host buffers; synchronous. */
TX_API int tx_compress_block_masked(int format, const uint8_t *rgba, uint32_t mask,
                                    const tx_params *params, uint8_t *output,
                                    size_t output_len);

/* Format::compress on device memory, stream-ordered.
 * src: width x height pixels of `channels` bytes each (4 = RGBA8 for every
 * format; 1 = R8 for BC4; 2 = RG8 for BC5 -- the 1-4 channel input of
 * README.md:42), rows src_pitch bytes apart.  output: output_len bytes, at
 * least tx_compressed_size(); the same full-block rule as tx_compress.
 * output must be aligned to the block size. */
TX_API int tx_compress_device(int format, const void *src, size_t src_pitch, int channels,
                              size_t width, size_t height, const tx_params *params,
                              void *output, size_t output_len, void *stream);

/* Format::compress_block_masked over many blocks on device memory,
 * stream-ordered.  blocks: nblocks x 64 bytes of RGBA8; masks: nblocks
 * uint32 (NULL = all 16 pixels valid); output: nblocks x block_size bytes,
 * aligned to the block size. */
TX_API int tx_compress_blocks_device(int format, const void *blocks, const uint32_t *masks,
                                     size_t nblocks, const tx_params *params, void *output,
                                     void *stream);

/* Format::decompress -- lib/src/lib.rs:124-156.  output: RGBA8, the rows of
 * pixels that output_len covers are written (as the reference chunks the
 * whole output).  data_len must cover every block those rows read. */
TX_API int tx_decompress(int format, const uint8_t *data, size_t data_len, size_t width,
                         size_t height, uint8_t *output, size_t output_len);

/* Format::decompress_block -- lib/src/lib.rs:240-277.  block_len >=
 * tx_block_size(format); rgba receives 64 bytes. */
TX_API int tx_decompress_block(int format, const uint8_t *block, size_t block_len,
                               uint8_t *rgba);

/* Format::decompress on device memory, stream-ordered.  output rows are
 * out_pitch bytes apart and hold width*4 bytes of RGBA8; height rows. */
TX_API int tx_decompress_device(int format, const void *data, size_t data_len, size_t width,
                                size_t height, void *output, size_t out_pitch, void *stream);

/* The CUDA error behind the last TX_ERR_CUDA returned on this thread
 * (a cudaError_t value), or 0. */
TX_API int tx_last_cuda_error(void);

/* Number of kernels this library has launched in this process (all
 * devices, all threads).  Used to account GPU work in benchmarks. */
TX_API uint64_t tx_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* TEXPRESSO_GB300_H */
