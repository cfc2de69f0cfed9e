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

/* ---------------------------------------------------------------------------
 * Batched form (no counterpart in the reference, which compresses one image
 * per call, lib/src/lib.rs:287): many textures / mip levels of mixed formats
 * and algorithms in one stream-ordered launch.  Each item is compressed
 * exactly as tx_compress_device would compress it. */

/* One texture level in device memory. */
typedef struct tx_batch_item {
    const void *src;      /* width x height pixels of `channels` bytes */
    size_t src_pitch;     /* bytes between rows */
    uint32_t width, height;
    int32_t format;       /* TX_FORMAT_* */
    int32_t channels;     /* 4 = RGBA8; 1 = R8 (BC4); 2 = RG8 (BC5) */
    tx_params params;
    void *dst;            /* tx_compressed_size(format, width, height) bytes, block-size aligned */
} tx_batch_item;

/* Launch shape of the two persistent kernels.  Zero fields take defaults. */
typedef struct tx_batch_tuning {
    int32_t team_lanes;            /* lanes per ClusterFit block: 16 or 32 */
    int32_t team_threads_per_cta;  /* threads per CTA of the ClusterFit kernel: 64..256 */
    int32_t team_ctas_per_sm;      /* persistent grid = SMs x this */
    int32_t team_blocks_per_unit;  /* ClusterFit blocks a team takes per queue pop */
    int32_t lane_ctas_per_sm;      /* RangeFit/BC4/BC5 kernel: persistent grid = SMs x this */
    int32_t lane_blocks_per_lane;  /* blocks per lane per queue pop (units of 32 x this) */
    int32_t team_blocks_in_flight; /* staging depth of the ClusterFit kernel: blocks whose pixels a team
                                    * holds or has requested, 1 (none ahead) to 3 (two ahead) */
} tx_batch_tuning;

typedef struct tx_batch tx_batch;  /* opaque plan; not thread-safe */

TX_API void tx_batch_default_tuning(tx_batch_tuning *tuning);

/* Validate the items and build the plan (allocates device memory for the
 * item table, the work queues and two counters).  Items are read at launch
 * time, so their buffers must stay valid while the plan is launched.  A level
 * of more than 2^31 - 1 blocks returns TX_ERR_INVALID_ARGUMENT. */
TX_API int tx_batch_create(const tx_batch_item *items, size_t nitems, const tx_batch_tuning *tuning,
                           tx_batch **batch);

/* Enqueue the whole batch on `stream` (a memset of the queue counters and
 * the persistent kernels, forked onto an internal second stream and joined
 * back).  Capturable in a CUDA graph; do not launch one plan concurrently
 * on two streams. */
TX_API int tx_batch_launch(tx_batch *batch, void *stream);

TX_API int tx_batch_set_tuning(tx_batch *batch, const tx_batch_tuning *tuning);
TX_API int tx_batch_get_tuning(const tx_batch *batch, tx_batch_tuning *tuning);
TX_API int tx_batch_info(const tx_batch *batch, size_t *nblocks, size_t *lane_units, size_t *team_units);

/* Time candidate launch shapes on this batch (coordinate descent, `repeats`
 * launches per candidate, CUDA events on `stream`), keep the fastest and
 * return it in *chosen (may be NULL).  Synchronises `stream`. */
TX_API int tx_batch_autotune(tx_batch *batch, void *stream, int repeats, tx_batch_tuning *chosen);

TX_API void tx_batch_destroy(tx_batch *batch);

/* Allocation-free batch launch.  No counterpart in the reference.  For
 * callers that must not have a library allocate device memory -- engines that
 * reserve the whole memory budget up front and hand it out through their own
 * allocator, or per-frame loops that cannot take the implicit synchronisation
 * of an allocation or free.  Compresses up to 256 texture levels to the same
 * output bytes as tx_batch_create + tx_batch_launch (and tx_compress_device),
 * but keeps the work queue in a fixed 1 MiB array of device memory that the
 * library declares statically (every GPU that loads the library holds it
 * until the process exits), so the call itself allocates nothing.  When the
 * default work units would overflow that array, the units grow (more blocks
 * per unit) until the queue fits, so the scheduling differs from
 * tx_batch_launch while the bytes do not.  The caller passes inputs and
 * outputs as in tx_batch_item.  More than 256 items, or a level of more than
 * 2^31 - 1 blocks, returns TX_ERR_INVALID_ARGUMENT.
 * Stream-ordered.  The first call on each device does a one-time set-up with
 * that device current (it looks up the array's device address); make that
 * first call before any stream capture.  All calls share the array, so calls
 * whose work overlaps on the GPU (other streams or threads) race: order them
 * on one stream. */
TX_API int tx_batch_launch_noalloc(const tx_batch_item *items, size_t nitems, void *stream);

/* Mip producer (the reference builds no mips, cli/src/main.rs:153): one level
 * step, next = max(1, size / 2) per axis, each output channel the 2x2 box
 * average (a+b+c+d+2)>>2 of the source with coordinates clamped at odd edges. */
typedef struct tx_mip_job {
    const void *src;
    size_t src_pitch;
    uint32_t width, height;  /* source level size */
    int32_t channels;        /* bytes per pixel, 1..4 */
    void *dst;
    size_t dst_pitch;
} tx_mip_job;

/* Number of levels of a full chain down to 1x1 (0 for an empty image). */
TX_API uint32_t tx_mip_count(uint32_t width, uint32_t height);

/* Produce one level for every job, stream-ordered, no allocation. */
TX_API int tx_mip_batch_device(const tx_mip_job *jobs, size_t njobs, void *stream);

/* ---------------------------------------------------------------------------
 * Serving form (no counterpart in the reference): a request loop that admits
 * compression jobs first-in first-out while the bytes they hold stay within a
 * budget and the device's free memory (cudaMemGetInfo, less 1 GiB of
 * headroom) covers them, takes their memory from a stream-ordered pool of its
 * own (trimmed when the server idles), batches every ready
 * job into each compression step (continuous batching: jobs that arrive while
 * others run join the next step; each job gets a round-robin share of every
 * step) and overlaps host<->device copies with compression.  A job's output
 * bytes are the same as tx_compress's for every level. */

/* Compressed bytes of a level chain: level 0 only (mips == 0) or every
 * box-filtered level down to 1x1 (mips != 0), concatenated level 0 first. */
TX_API size_t tx_chain_compressed_size(int format, uint32_t width, uint32_t height, int mips);

typedef struct tx_server_config {
    size_t memory_budget;     /* most device bytes admitted jobs may hold; default 40 GiB */
    uint32_t step_blocks;     /* blocks per compression step; default 1 Mi */
    uint32_t min_share;       /* blocks a ready job gets per step at least; default 16 Ki */
    tx_batch_tuning tuning;   /* launch shape of the step kernels (zero fields: defaults) */
} tx_server_config;

typedef struct tx_server_request {
    const uint8_t *rgba;      /* host RGBA8, width*height*4 bytes, valid until the job completes */
    uint32_t width, height;
    int32_t format;           /* TX_FORMAT_* */
    tx_params params;
    int32_t mips;             /* non-zero: compress the full mip chain */
    uint8_t *output;          /* host, tx_chain_compressed_size() bytes, written on completion */
    size_t output_len;
} tx_server_request;

typedef struct tx_server_result {
    int32_t status;           /* TX_OK or the error that ended the job */
    uint32_t levels, steps;   /* levels compressed, compression steps the job took part in */
    uint64_t blocks;
    double latency_us;        /* submit -> output written to host */
    double queue_us;          /* submit -> admitted into device memory */
} tx_server_result;

typedef struct tx_server_stats {
    uint64_t submitted, completed, steps;
    size_t memory_budget;     /* the configured budget */
    size_t held_high_water;   /* most device bytes admitted jobs held at once */
    double busy_us;           /* device time of the compression steps so far (CUDA events) */
    uint64_t hbm_deferrals;   /* jobs whose admission waited for free device memory */
} tx_server_stats;

typedef struct tx_server tx_server;

TX_API void tx_server_default_config(tx_server_config *config);
/* Allocate the arena and start the worker thread on the current device. */
TX_API int tx_server_create(const tx_server_config *config, tx_server **server);
/* Queue a job (thread-safe).  A job larger than the whole budget returns
 * TX_ERR_OUT_OF_MEMORY at once. */
TX_API int tx_server_submit(tx_server *server, const tx_server_request *request, uint64_t *id);
/* Wait for a job (timeout_ms < 0: no limit) and release it; returns the
 * job's status, or TX_ERR_TIMEOUT with the job still pending. */
TX_API int tx_server_wait(tx_server *server, uint64_t id, int timeout_ms, tx_server_result *result);
/* Cancel a job that has not been admitted into device memory yet: returns
 * TX_OK and its wait then returns TX_ERR_CANCELLED; a job already admitted
 * returns TX_ERR_BUSY and completes normally. */
TX_API int tx_server_cancel(tx_server *server, uint64_t id);
TX_API int tx_server_get_stats(tx_server *server, tx_server_stats *stats);
/* Finish every queued job, then stop the worker and free the arena. */
TX_API void tx_server_destroy(tx_server *server);

/* ---------------------------------------------------------------------------
 * DDS container (host only; cli/src/main.rs:143-196 writes and reads DDS
 * through the ddsfile crate).  A DDS file is TX_DDS_HEADER_BYTES of header
 * followed by the compressed levels, level 0 first. */
#define TX_DDS_HEADER_BYTES 148

/* Write the magic, DDS_HEADER and DDS_HEADER_DXT10 the CLI writes
 * (cli/src/main.rs:143-164): DXGI BC1/BC2/BC3 UNORM_SRGB, BC4/BC5 UNORM,
 * Texture2D, alpha mode premultiplied for BC1 and straight otherwise.
 * mip_levels <= 1 writes no mip count (the CLI's case). */
TX_API int tx_dds_write_header(int format, uint32_t width, uint32_t height, uint32_t mip_levels,
                               uint8_t *out, size_t out_len, size_t *written);

/* Read a DDS header as cli/src/main.rs:167-196 does: a DX10 header with the
 * DXGI formats above and Texture2D, or a legacy DXT1/DXT3/DXT5 FourCC.
 * Returns TX_ERR_INVALID_FORMAT where the CLI panics on the format. */
TX_API int tx_dds_parse(const uint8_t *data, size_t len, int *format, uint32_t *width, uint32_t *height,
                        uint32_t *mip_levels, size_t *data_offset);

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
