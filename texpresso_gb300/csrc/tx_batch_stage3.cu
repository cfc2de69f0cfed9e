// tx_batch_stage3.cu -- the batch team kernels with 3 block(s) in flight per
// team (tx_batch_teams.cuh), in a translation unit of their own.
#include "tx_batch_teams.cuh"

namespace tx {

template cudaError_t launch_team_class<3>(int team, int c, const BatchQueue &q, uint32_t grid, int threads,
                                          cudaStream_t st);
template cudaError_t prepare_team_class_kernels<3>();
template cudaError_t upload_stage_tables<3>(const uint32_t lut[4][256][2]);

}  // namespace tx
