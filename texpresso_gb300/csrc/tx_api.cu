// tx_api.cu -- the C ABI (include/texpresso_gb300.h): argument checks that
// mirror the reference's panics, per-device state, and the host-buffer path
// that streams an image through the GPU in bands of block rows so that the
// host->device copy of one band overlaps the kernel of the previous one.
#include "texpresso_gb300.h"
#include "tx_device.cuh"
#include "tx_internal.h"

#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstring>
#include <mutex>

namespace tx {

static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

}  // namespace tx

namespace {

thread_local int t_last_cuda = 0;

constexpr int kMaxDevices = 64;
constexpr int kStreams = 3;

struct DeviceState {
    std::mutex mu;                      // serialises host-buffer calls on this device
    std::atomic<int> ready{0};          // tables uploaded
    cudaStream_t streams[kStreams] = {};
    cudaEvent_t joined[kStreams] = {};  // streams 1.. joined into stream 0 at the end of a call
    uint8_t *d_in = nullptr;
    size_t in_cap = 0;
    uint8_t *d_out = nullptr;
    size_t out_cap = 0;
    int sm_count = 0;
};

DeviceState g_dev[kMaxDevices];
std::mutex g_init_mu;

int fail(cudaError_t e) {
    t_last_cuda = (int)e;
    if (e == cudaErrorMemoryAllocation) return TX_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return TX_ERR_NO_DEVICE;
    return TX_ERR_CUDA;
}

// Single-colour tables of lib/src/colourfit/single_lut.rs, produced by the
// generator they come from (libsquish's): for every endpoint pair, in order
// (v1 outer, v2 inner), the 8-bit values hit by code 0 and by the first
// interpolant get error 0 (first pair wins); then errors relax from the right
// and the left neighbour until nothing changes.
void build_single_table(int bits, int colours, uint32_t out[256][2]) {
    int start[256][2], end[256][2], err[256][2];
    for (int t = 0; t < 256; ++t)
        for (int k = 0; k < 2; ++k) { start[t][k] = 0; end[t][k] = 0; err[t][k] = 255; }
    const int n = 1 << bits;
    for (int v1 = 0; v1 < n; ++v1)
        for (int v2 = 0; v2 < n; ++v2) {
            const int a = (v1 << (8 - bits)) | (v1 >> (2 * bits - 8));
            const int b = (v2 << (8 - bits)) | (v2 >> (2 * bits - 8));
            const int target[2] = {a, colours == 3 ? (a + b) / 2 : (2 * a + b) / 3};
            for (int k = 0; k < 2; ++k) {
                const int t = target[k];
                if (err[t][k] != 0) { start[t][k] = v1; end[t][k] = v2; err[t][k] = 0; }
            }
        }
    bool changed = true;
    while (changed) {
        changed = false;
        for (int k = 0; k < 2; ++k)
            for (int t = 0; t < 256; ++t) {
                for (int nb = 0; nb < 2; ++nb) {
                    const int u = nb == 0 ? t + 1 : t - 1;
                    if (u < 0 || u > 255) continue;
                    if (err[t][k] > err[u][k] + 1) {
                        start[t][k] = start[u][k];
                        end[t][k] = end[u][k];
                        err[t][k] = err[u][k] + 1;
                        changed = true;
                    }
                }
            }
    }
    for (int t = 0; t < 256; ++t)
        for (int k = 0; k < 2; ++k)
            out[t][k] = (uint32_t)start[t][k] | ((uint32_t)end[t][k] << 8) | ((uint32_t)err[t][k] << 16);
}

int get_device(int *dev) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        t_last_cuda = (int)e;
        return TX_ERR_NO_DEVICE;
    }
    if ((e = cudaGetDevice(dev)) != cudaSuccess) return fail(e);
    if (*dev < 0 || *dev >= kMaxDevices) return TX_ERR_NO_DEVICE;
    return TX_OK;
}

// Upload tables and create streams for the current device (once).
int ensure_ready(DeviceState **out) {
    int dev = 0;
    int rc = get_device(&dev);
    if (rc != TX_OK) return rc;
    DeviceState &d = g_dev[dev];
    *out = &d;
    if (d.ready.load(std::memory_order_acquire)) return TX_OK;
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (d.ready.load(std::memory_order_relaxed)) return TX_OK;
    static uint32_t lut[4][256][2];
    build_single_table(5, 3, lut[0]);
    build_single_table(6, 3, lut[1]);
    build_single_table(5, 4, lut[2]);
    build_single_table(6, 4, lut[3]);
    cudaError_t e = tx::upload_colour_tables(lut);
    if (e != cudaSuccess) return fail(e);
    if ((e = tx::upload_batch_tables(lut)) != cudaSuccess) return fail(e);
    for (int s = 0; s < kStreams; ++s) {
        if ((e = cudaStreamCreateWithFlags(&d.streams[s], cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
        if ((e = cudaEventCreateWithFlags(&d.joined[s], cudaEventDisableTiming)) != cudaSuccess) return fail(e);
    }
    if ((e = cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return fail(e);
    d.ready.store(1, std::memory_order_release);
    return TX_OK;
}

cudaError_t grow(uint8_t **buf, size_t *cap, size_t need) {
    if (need <= *cap) return cudaSuccess;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    size_t sz = need + (need >> 3);
    sz = (sz + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(buf, sz);
    if (e == cudaSuccess) *cap = sz;
    return e;
}

bool valid_format(int f) { return f >= TX_FORMAT_BC1 && f <= TX_FORMAT_BC5; }

int check_params(int format, const tx_params *p, tx::DevParams *dp, int *algorithm) {
    tx_params def;
    tx_params_default(&def);
    if (!p) p = &def;
    if (p->algorithm < TX_RANGE_FIT || p->algorithm > TX_ITERATIVE_CLUSTER_FIT) return TX_ERR_INVALID_ARGUMENT;
    for (int c = 0; c < 3; ++c) dp->w[c] = p->weights[c];
    dp->alpha_weighted = p->weigh_colour_by_alpha ? 1 : 0;
    *algorithm = p->algorithm;
    (void)format;
    return TX_OK;
}

bool mul_overflows(size_t a, size_t b, size_t *r) {
    if (a != 0 && b > SIZE_MAX / a) return true;
    *r = a * b;
    return false;
}

cudaError_t launch_any(int format, int algorithm, const tx::SrcDesc &src, const tx::DevParams &dp, uint8_t *out,
                       size_t nblocks, cudaStream_t st) {
    tx::LaunchCfg cfg;
    if (format == TX_FORMAT_BC4 || format == TX_FORMAT_BC5) return tx::launch_alpha(format, src, out, nblocks, st, cfg);
    return tx::launch_colour(format, algorithm, src, dp, out, nblocks, st, cfg);
}

// Shared validation of Format::compress arguments (lib/src/lib.rs:287-303).
int check_compress(int format, size_t width, size_t height, size_t output_len, size_t *nblocks) {
    if (!valid_format(format)) return TX_ERR_INVALID_FORMAT;
    if (width == 0) return TX_ERR_INVALID_ARGUMENT;  // chunk size 0 panics
    const size_t bs = tx_block_size(format);
    if (output_len < tx_compressed_size(format, width, height)) return TX_ERR_OUTPUT_TOO_SMALL;
    if (output_len % bs != 0) return TX_ERR_INVALID_ARGUMENT;  // trailing partial block panics
    *nblocks = output_len / bs;
    const size_t bw = tx_num_blocks(width);
    if (width > 0xFFFFFFF0u || height > 0xFFFFFFF0u || *nblocks / bw > 0x3FFFFFFFu) return TX_ERR_INVALID_ARGUMENT;
    return TX_OK;
}

}  // namespace

int tx_internal_ensure_device() {
    DeviceState *d = nullptr;
    return ensure_ready(&d);
}

void tx_internal_set_last_cuda_error(int err) { t_last_cuda = err; }

extern "C" {

void tx_params_default(tx_params *p) {
    if (!p) return;
    p->algorithm = TX_CLUSTER_FIT;
    p->weights[0] = 0.2126f;
    p->weights[1] = 0.7152f;
    p->weights[2] = 0.0722f;
    p->weigh_colour_by_alpha = 0;
}

const char *tx_status_string(int status) {
    switch (status) {
    case TX_OK: return "ok";
    case TX_ERR_INVALID_FORMAT: return "invalid format";
    case TX_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TX_ERR_OUTPUT_TOO_SMALL: return "output buffer too small";
    case TX_ERR_INPUT_TOO_SMALL: return "input buffer too small";
    case TX_ERR_CUDA: return "CUDA error";
    case TX_ERR_NO_DEVICE: return "no usable CUDA device";
    case TX_ERR_TIMEOUT: return "timed out";
    case TX_ERR_OUT_OF_MEMORY: return "out of device memory";
    case TX_ERR_MISALIGNED: return "misaligned buffer";
    case TX_ERR_BUSY: return "busy";
    case TX_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
    }
}

size_t tx_num_blocks(size_t size) { return (size + 3) / 4; }

size_t tx_block_size(int format) {
    if (!valid_format(format)) return 0;
    return (format == TX_FORMAT_BC1 || format == TX_FORMAT_BC4) ? 8 : 16;
}

size_t tx_compressed_size(int format, size_t width, size_t height) {
    return tx_num_blocks(width) * tx_num_blocks(height) * tx_block_size(format);
}

int tx_last_cuda_error(void) { return t_last_cuda; }

uint64_t tx_kernel_launch_count(void) { return tx::g_launches.load(std::memory_order_relaxed); }

int tx_compress(int format, const uint8_t *rgba, size_t rgba_len, size_t width, size_t height,
                const tx_params *params, uint8_t *output, size_t output_len) {
    size_t nblocks = 0;
    int rc = check_compress(format, width, height, output_len, &nblocks);
    if (rc != TX_OK) return rc;
    tx::DevParams dp;
    int algorithm = 0;
    if ((rc = check_params(format, params, &dp, &algorithm)) != TX_OK) return rc;
    size_t in_bytes = 0;
    if (mul_overflows(width, height, &in_bytes) || mul_overflows(in_bytes, 4, &in_bytes)) return TX_ERR_INVALID_ARGUMENT;
    if (rgba_len < in_bytes || (in_bytes && !rgba)) return TX_ERR_INPUT_TOO_SMALL;
    if (nblocks && !output) return TX_ERR_INVALID_ARGUMENT;
    if (nblocks == 0) return TX_OK;
    DeviceState *d = nullptr;
    if ((rc = ensure_ready(&d)) != TX_OK) return rc;
    std::lock_guard<std::mutex> lk(d->mu);
    struct Range {
        Range() { nvtxRangePushA("tx_compress"); }
        ~Range() { nvtxRangePop(); }
    } range;
    cudaError_t e;
    if ((e = grow(&d->d_in, &d->in_cap, in_bytes ? in_bytes : 16)) != cudaSuccess) return fail(e);
    if ((e = grow(&d->d_out, &d->out_cap, output_len)) != cudaSuccess) return fail(e);

    const size_t bs = tx_block_size(format), bw = tx_num_blocks(width);
    const size_t rows = (nblocks + bw - 1) / bw;  // output block rows (may exceed the image)
    const size_t pitch = 4 * width;
    // Bands of block rows, each copied in, compressed and copied out on one of
    // the streams, so the copies of one band overlap the kernels of others.
    // Large images taper the bands (weights 1 4 8 8 8 8 8 4 1 of 50): the
    // first band's upload and the last band's download are the only copies
    // nothing overlaps, so they are kept small.
    static const int kTaper[] = {1, 4, 8, 8, 8, 8, 8, 4, 1};
    constexpr int kTaperBands = 9, kTaperSum = 50;
    const bool taper = rows >= 2 * kTaperSum;
    size_t nbands = taper ? kTaperBands : rows / 32;
    if (nbands < 1) nbands = 1;
    if (nbands > 8 && !taper) nbands = 8;
    const size_t band_rows = (rows + nbands - 1) / nbands;
    size_t done_w = 0;
    for (size_t r0 = 0, band = 0; r0 < rows; ++band) {
        size_t r1;
        if (taper) {
            done_w += (size_t)kTaper[band];
            r1 = band + 1 == (size_t)kTaperBands ? rows : rows * done_w / kTaperSum;
        } else {
            r1 = r0 + band_rows < rows ? r0 + band_rows : rows;
        }
        cudaStream_t st = d->streams[band % kStreams];
        // input rows of this band
        const size_t y0 = 4 * r0, y1 = (4 * r1 < height) ? 4 * r1 : height;
        if (y0 < y1) {
            if ((e = cudaMemcpyAsync(d->d_in + y0 * pitch, rgba + y0 * pitch, (y1 - y0) * pitch,
                                     cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return fail(e);
        }
        const size_t b0 = r0 * bw, b1 = (r1 * bw < nblocks) ? r1 * bw : nblocks;
        tx::SrcDesc src;
        src.base = d->d_in + (y0 < height ? y0 : 0) * pitch;
        src.masks = nullptr;
        src.pitch = pitch;
        src.width = (uint32_t)width;
        src.height = (uint32_t)(height > y0 ? height - y0 : 0);
        tx::set_blocks_wide(src, (uint32_t)bw);
        src.channels = 4;
        src.vec16 = (pitch % 16 == 0) ? 1 : 0;
        src.mode = 0;
        if ((e = launch_any(format, algorithm, src, dp, d->d_out + b0 * bs, b1 - b0, st)) != cudaSuccess) return fail(e);
        if ((e = cudaMemcpyAsync(output + b0 * bs, d->d_out + b0 * bs, (b1 - b0) * bs, cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess)
            return fail(e);
        r0 = r1;
    }
    // one wait: the other streams join stream 0
    for (int s = 1; s < kStreams; ++s) {
        if ((e = cudaEventRecord(d->joined[s], d->streams[s])) != cudaSuccess) return fail(e);
        if ((e = cudaStreamWaitEvent(d->streams[0], d->joined[s], 0)) != cudaSuccess) return fail(e);
    }
    if ((e = cudaStreamSynchronize(d->streams[0])) != cudaSuccess) return fail(e);
    return TX_OK;
}

int tx_compress_block_masked(int format, const uint8_t *rgba, uint32_t mask, const tx_params *params,
                             uint8_t *output, size_t output_len) {
    if (!valid_format(format)) return TX_ERR_INVALID_FORMAT;
    if (!rgba || !output) return TX_ERR_INVALID_ARGUMENT;
    const size_t bs = tx_block_size(format);
    if (output_len < bs) return TX_ERR_OUTPUT_TOO_SMALL;
    tx::DevParams dp;
    int algorithm = 0;
    int rc = check_params(format, params, &dp, &algorithm);
    if (rc != TX_OK) return rc;
    DeviceState *d = nullptr;
    if ((rc = ensure_ready(&d)) != TX_OK) return rc;
    std::lock_guard<std::mutex> lk(d->mu);
    cudaError_t e;
    if ((e = grow(&d->d_in, &d->in_cap, 128)) != cudaSuccess) return fail(e);
    if ((e = grow(&d->d_out, &d->out_cap, 16)) != cudaSuccess) return fail(e);
    uint8_t staging[68];
    std::memcpy(staging, rgba, 64);
    std::memcpy(staging + 64, &mask, 4);
    cudaStream_t st = d->streams[0];
    if ((e = cudaMemcpyAsync(d->d_in, staging, 68, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e);
    tx::SrcDesc src;
    std::memset(&src, 0, sizeof(src));
    src.base = d->d_in;
    src.masks = reinterpret_cast<const uint32_t *>(d->d_in + 64);
    src.channels = 4;
    src.mode = 1;
    if ((e = launch_any(format, algorithm, src, dp, d->d_out, 1, st)) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpyAsync(output, d->d_out, bs, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    return TX_OK;
}

int tx_compress_device(int format, const void *src_ptr, size_t src_pitch, int channels, size_t width, size_t height,
                       const tx_params *params, void *output, size_t output_len, void *stream) {
    size_t nblocks = 0;
    int rc = check_compress(format, width, height, output_len, &nblocks);
    if (rc != TX_OK) return rc;
    tx::DevParams dp;
    int algorithm = 0;
    if ((rc = check_params(format, params, &dp, &algorithm)) != TX_OK) return rc;
    const bool ok_ch = channels == 4 || (channels == 1 && format == TX_FORMAT_BC4) ||
                       (channels == 2 && format == TX_FORMAT_BC5);
    if (!ok_ch) return TX_ERR_INVALID_ARGUMENT;
    if (src_pitch < (size_t)channels * width) return TX_ERR_INVALID_ARGUMENT;
    const size_t bs = tx_block_size(format);
    if (nblocks && (!output || (reinterpret_cast<uintptr_t>(output) % bs) != 0)) return output ? TX_ERR_MISALIGNED : TX_ERR_INVALID_ARGUMENT;
    if (height && !src_ptr) return TX_ERR_INVALID_ARGUMENT;
    if (nblocks == 0) return TX_OK;
    DeviceState *d = nullptr;
    if ((rc = ensure_ready(&d)) != TX_OK) return rc;
    tx::SrcDesc src;
    src.base = static_cast<const uint8_t *>(src_ptr);
    src.masks = nullptr;
    src.pitch = src_pitch;
    src.width = (uint32_t)width;
    src.height = (uint32_t)height;
    tx::set_blocks_wide(src, (uint32_t)tx_num_blocks(width));
    src.channels = channels;
    const size_t vec_align = channels == 4 ? 16 : (size_t)channels * 4;
    src.vec16 = ((reinterpret_cast<uintptr_t>(src_ptr) % vec_align) == 0 && (src_pitch % vec_align) == 0) ? 1 : 0;
    src.mode = 0;
    cudaError_t e = launch_any(format, algorithm, src, dp, static_cast<uint8_t *>(output), nblocks,
                               static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TX_OK : fail(e);
}

int tx_compress_blocks_device(int format, const void *blocks, const uint32_t *masks, size_t nblocks,
                              const tx_params *params, void *output, void *stream) {
    if (!valid_format(format)) return TX_ERR_INVALID_FORMAT;
    tx::DevParams dp;
    int algorithm = 0;
    int rc = check_params(format, params, &dp, &algorithm);
    if (rc != TX_OK) return rc;
    if (nblocks == 0) return TX_OK;
    if (!blocks || !output) return TX_ERR_INVALID_ARGUMENT;
    const size_t bs = tx_block_size(format);
    if ((reinterpret_cast<uintptr_t>(output) % bs) != 0 || (reinterpret_cast<uintptr_t>(blocks) % 16) != 0 ||
        (reinterpret_cast<uintptr_t>(masks) % 4) != 0)
        return TX_ERR_MISALIGNED;
    DeviceState *d = nullptr;
    if ((rc = ensure_ready(&d)) != TX_OK) return rc;
    tx::SrcDesc src;
    std::memset(&src, 0, sizeof(src));
    src.base = static_cast<const uint8_t *>(blocks);
    src.masks = masks;
    src.channels = 4;
    src.mode = 1;
    cudaError_t e = launch_any(format, algorithm, src, dp, static_cast<uint8_t *>(output), nblocks,
                               static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TX_OK : fail(e);
}

int tx_decompress(int format, const uint8_t *data, size_t data_len, size_t width, size_t height, uint8_t *output,
                  size_t output_len) {
    if (!valid_format(format)) return TX_ERR_INVALID_FORMAT;
    if (width == 0) return TX_ERR_INVALID_ARGUMENT;
    const size_t bs = tx_block_size(format), bw = tx_num_blocks(width);
    const size_t row_bytes = width * 16;
    const size_t rows = (output_len + row_bytes - 1) / row_bytes;  // chunks of the output
    if (rows == 0) return TX_OK;
    if (rows * bw * bs > data_len) return TX_ERR_INPUT_TOO_SMALL;
    // every pixel of the image that falls in a chunk must fit the output
    const size_t img_rows = (4 * rows < height) ? 4 * rows : height;
    if (img_rows > 0 && img_rows * width * 4 > output_len) return TX_ERR_OUTPUT_TOO_SMALL;
    if (!data || !output) return TX_ERR_INVALID_ARGUMENT;
    DeviceState *d = nullptr;
    int rc = ensure_ready(&d);
    if (rc != TX_OK) return rc;
    std::lock_guard<std::mutex> lk(d->mu);
    cudaError_t e;
    const size_t in_bytes = rows * bw * bs;
    if ((e = grow(&d->d_in, &d->in_cap, in_bytes)) != cudaSuccess) return fail(e);
    if ((e = grow(&d->d_out, &d->out_cap, output_len)) != cudaSuccess) return fail(e);
    cudaStream_t st = d->streams[0];
    if ((e = cudaMemcpyAsync(d->d_in, data, in_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e);
    if ((e = tx::launch_decode(format, d->d_in, bw, rows, width, height, d->d_out, width * 4, output_len, st)) !=
        cudaSuccess)
        return fail(e);
    // every pixel of the first img_rows rows is written; bytes past them stay untouched
    const size_t written = img_rows * width * 4;
    if (written && (e = cudaMemcpyAsync(output, d->d_out, written, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    return TX_OK;
}

int tx_decompress_block(int format, const uint8_t *block, size_t block_len, uint8_t *rgba) {
    if (!valid_format(format)) return TX_ERR_INVALID_FORMAT;
    if (!block || !rgba) return TX_ERR_INVALID_ARGUMENT;
    const size_t bs = tx_block_size(format);
    if (block_len < bs) return TX_ERR_INPUT_TOO_SMALL;
    DeviceState *d = nullptr;
    int rc = ensure_ready(&d);
    if (rc != TX_OK) return rc;
    std::lock_guard<std::mutex> lk(d->mu);
    cudaError_t e;
    if ((e = grow(&d->d_in, &d->in_cap, 16)) != cudaSuccess) return fail(e);
    if ((e = grow(&d->d_out, &d->out_cap, 64)) != cudaSuccess) return fail(e);
    cudaStream_t st = d->streams[0];
    if ((e = cudaMemcpyAsync(d->d_in, block, bs, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e);
    if ((e = tx::launch_decode(format, d->d_in, 1, 1, 4, 4, d->d_out, 16, 64, st)) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpyAsync(rgba, d->d_out, 64, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return fail(e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e);
    return TX_OK;
}

int tx_decompress_device(int format, const void *data, size_t data_len, size_t width, size_t height, void *output,
                         size_t out_pitch, void *stream) {
    if (!valid_format(format)) return TX_ERR_INVALID_FORMAT;
    if (width == 0) return TX_ERR_INVALID_ARGUMENT;
    const size_t bs = tx_block_size(format), bw = tx_num_blocks(width), bh = tx_num_blocks(height);
    if (bw * bh * bs > data_len) return TX_ERR_INPUT_TOO_SMALL;
    if (out_pitch < width * 4) return TX_ERR_INVALID_ARGUMENT;
    if (bh == 0) return TX_OK;
    if (!data || !output) return TX_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(data) % 8) != 0) return TX_ERR_MISALIGNED;
    DeviceState *d = nullptr;
    int rc = ensure_ready(&d);
    if (rc != TX_OK) return rc;
    cudaError_t e = tx::launch_decode(format, static_cast<const uint8_t *>(data), bw, bh, width, height,
                                      static_cast<uint8_t *>(output), out_pitch, out_pitch * height,
                                      static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? TX_OK : fail(e);
}

}  // extern "C"
