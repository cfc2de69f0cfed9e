// tx_alpha.cu -- BC4 / BC5 single-texture kernel (device code in tx_alpha.cuh).
//
// One thread per 4x4 block.  The codebook search runs four pixels per 32-bit
// word (tx_device.cuh: encode_bc3_alpha).
#include "tx_alpha.cuh"
#include "tx_internal.h"

namespace tx {

template <int FMT, int CH>
__global__ void __launch_bounds__(256) k_alpha(SrcDesc src, uint8_t *__restrict__ out, size_t nblocks) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks; b += stride)
        alpha_block<FMT, CH>(src, b, out);
}

template <int FMT, int CH>
static cudaError_t launch_t(const SrcDesc &src, uint8_t *out, size_t nblocks, cudaStream_t st, const LaunchCfg &cfg) {
    const int threads = 256;
    size_t grid = (nblocks + threads - 1) / threads;
    if (grid > cfg.max_ctas) grid = cfg.max_ctas;
    if (grid == 0) grid = 1;
    k_alpha<FMT, CH><<<(unsigned)grid, threads, 0, st>>>(src, out, nblocks);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_alpha(int fmt, const SrcDesc &src, uint8_t *out, size_t nblocks, cudaStream_t st,
                         const LaunchCfg &cfg) {
    if (nblocks == 0) return cudaSuccess;
    if (fmt == BC4) {
        if (src.channels == 4) return launch_t<BC4, 4>(src, out, nblocks, st, cfg);
        if (src.channels == 1) return launch_t<BC4, 1>(src, out, nblocks, st, cfg);
    } else if (fmt == BC5) {
        if (src.channels == 4) return launch_t<BC5, 4>(src, out, nblocks, st, cfg);
        if (src.channels == 2) return launch_t<BC5, 2>(src, out, nblocks, st, cfg);
    }
    return cudaErrorInvalidValue;
}

}  // namespace tx
