// tx_batch_internal.h -- device descriptors and the queue launcher shared by
// the batch plans (tx_batch.cu) and the serving loop (tx_server.cu).
#pragma once
#include "texpresso_gb300.h"
#include "tx_device.cuh"

namespace tx {

enum UnitKind : int32_t { KIND_ALPHA = 0, KIND_RANGE = 1, KIND_CLUSTER = 2, KIND_CLUSTER_ITER = 3 };

// Most blocks one batched level may have: block numbers, a unit's first block
// plus its span, and nblocks + span - 1 then stay below 2^32 for every span
// the plans use.
constexpr uint32_t kMaxBatchLevelBlocks = 0x7FFFFFFFu;

struct BatchItem {
    SrcDesc src;
    DevParams prm;
    uint8_t *dst;
    uint32_t nblocks;
    int32_t format;
    int32_t kind;
    int32_t channels;
};

struct BatchQueue {
    const BatchItem *items;
    const uint2 *units;     // (item, first block)
    uint32_t nunits;
    uint32_t *counter;
    uint32_t per_unit;      // lane units: blocks per lane; team units: blocks per unit
};

// Team units are grouped by class, each drained by its own kernel
// instantiation (so each gets the registers its code needs): class =
// (iterative ? 0 : 3) + format (BC1, BC2, BC3), iterative classes first.
constexpr int kTeamClasses = 6;
constexpr int kBatchCounters = 1 + kTeamClasses;  // lane queue, then one per team class

__host__ __device__ inline int team_class(int format, int kind) {
    return (kind == KIND_CLUSTER_ITER ? 0 : 3) + format;
}

// Fill a device descriptor from a validated public item.
void fill_batch_item(const tx_batch_item &it, BatchItem *d);

// Enqueue the persistent kernels of one team queue whose units are grouped by
// class (team_counts[c] units of class c, in class order) on `st`, one kernel
// per non-empty class, one after another.  counters[c] belongs to class c and
// must be zero when its kernel starts.
cudaError_t launch_team_classes(const BatchItem *d_items, const uint2 *d_team,
                                const uint32_t (&team_counts)[kTeamClasses], uint32_t team_blocks_per_unit,
                                uint32_t *counters, int sm_count, const tx_batch_tuning &tuning, cudaStream_t st);

// Raise the shared-memory limit of every team kernel with 32-lane teams on
// the current device (done by a plain launch on first use otherwise).
cudaError_t prepare_team_kernels();

// The team kernels with STAGE blocks in flight per team (1-3), one
// translation unit each (tx_batch_stage<STAGE>.cu, tx_batch_teams.cuh):
// launch the kernel of class c (see team_class) with `team` lanes per block,
// raise their shared-memory limits, and upload that unit's constant tables.
template <int STAGE>
cudaError_t launch_team_class(int team, int c, const BatchQueue &q, uint32_t grid, int threads, cudaStream_t st);
template <int STAGE>
cudaError_t prepare_team_class_kernels();
template <int STAGE>
cudaError_t upload_stage_tables(const uint32_t lut[4][256][2]);

// Enqueue the lane kernel and the team kernels over device-resident queues on
// `st` (sequentially).  counters[0 .. kBatchCounters) must be zero when the
// kernels start.
cudaError_t launch_batch_queues(const BatchItem *d_items, const uint2 *d_lane, uint32_t n_lane,
                                uint32_t lane_blocks_per_lane, const uint2 *d_team,
                                const uint32_t (&team_counts)[kTeamClasses], uint32_t team_blocks_per_unit,
                                uint32_t *d_counters, int sm_count, const tx_batch_tuning &tuning, cudaStream_t st);

}  // namespace tx
