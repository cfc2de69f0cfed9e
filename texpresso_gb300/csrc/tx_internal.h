// tx_internal.h -- declarations shared between the kernel translation units
// and the C ABI implementation (not part of the public interface).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace tx {

struct SrcDesc;
struct DevParams;

// Launch shape chosen per call (defaults, or the autotuner's pick).
struct LaunchCfg {
    size_t max_ctas = 1u << 30;  // cap on the grid (persistent launches use SMs x occupancy)
    int cluster_team = 32;       // lanes per 4x4 block in the ClusterFit kernel: 16 or 32
    int cluster_threads = 256;   // threads per CTA of the ClusterFit kernel
    int blocks_per_thread = 1;   // BC4/BC5 blocks handled by one thread
};

void note_launch();

// tx_colour.cu
cudaError_t upload_colour_tables(const uint32_t lut[4][256][2]);
cudaError_t launch_colour(int fmt, int algorithm, const SrcDesc &src, const DevParams &prm, uint8_t *out,
                          size_t nblocks, cudaStream_t st, const LaunchCfg &cfg);
size_t cluster_smem_bytes(int team, int threads);

// tx_batch.cu
cudaError_t upload_batch_tables(const uint32_t lut[4][256][2]);

// tx_alpha.cu
cudaError_t launch_alpha(int fmt, const SrcDesc &src, uint8_t *out, size_t nblocks, cudaStream_t st,
                         const LaunchCfg &cfg);

// tx_decode.cu
cudaError_t launch_decode(int fmt, const uint8_t *data, size_t blocks_wide, size_t block_rows, size_t width,
                          size_t height, uint8_t *out, size_t out_pitch, size_t out_len, cudaStream_t st);

}  // namespace tx

// tx_api.cu: shared device bookkeeping for every entry point
int tx_internal_ensure_device();                // tables uploaded on the current device
void tx_internal_set_last_cuda_error(int err);  // for tx_last_cuda_error()
