// tx_batch_internal.h -- device descriptors and the queue launcher shared by
// the batch plans (tx_batch.cu) and the serving loop (tx_server.cu).
#pragma once
#include "texpresso_gb300.h"
#include "tx_device.cuh"

namespace tx {

enum UnitKind : int32_t { KIND_ALPHA = 0, KIND_RANGE = 1, KIND_CLUSTER = 2, KIND_CLUSTER_ITER = 3 };

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

// Fill a device descriptor from a validated public item.
void fill_batch_item(const tx_batch_item &it, BatchItem *d);

// Enqueue the two persistent kernels over device-resident queues on `st`
// (sequentially).  counters[0..1] must be zero when the kernels start.
cudaError_t launch_batch_queues(const BatchItem *d_items, const uint2 *d_lane, uint32_t n_lane,
                                uint32_t lane_blocks_per_lane, const uint2 *d_team, uint32_t n_team,
                                uint32_t team_blocks_per_unit, uint32_t *d_counters, int sm_count,
                                const tx_batch_tuning &tuning, cudaStream_t st);

}  // namespace tx
