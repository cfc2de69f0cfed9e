// tx_batch.cu -- many textures (and their mip levels) in one stream-ordered,
// CUDA-graph-capturable launch.
//
// A plan (tx_batch) holds, in device memory, one descriptor per texture level
// and two work queues of "units" (a run of blocks of one level):
//   lane units  RangeFit, BC4, BC5 -- thread-per-block code; a warp pops a unit
//               of 32 x U blocks (U = blocks per lane) and each lane encodes
//               every 32nd block of it;
//   team units  ClusterFit, IterativeClusterFit -- a team of 32 lanes encodes
//               the unit's C blocks one after another.
// Each queue is drained by persistent kernels (grid = SMs x CTAs per SM);
// warps pop units with one atomicAdd on a queue counter, so uneven levels
// (4x4 mips next to 4096x4096 bases) balance themselves.  Team units are
// grouped by class (format x iterative or single-pass), iterative classes
// first, and each class is drained by its own kernel instantiation, so each
// gets the register budget its code needs.  The lane kernel and the team
// kernels run on two streams forked from the caller's stream; a launch is a
// memset of the counters plus the kernels, so it can be captured in a CUDA
// graph and replayed.
//
// The per-block code is the single-texture code (tx_colour.cuh,
// tx_alpha.cuh), so a batch produces exactly the bytes of per-texture calls.
#include "texpresso_gb300.h"
#include "tx_alpha.cuh"
#include "tx_colour.cuh"
#include "tx_internal.h"
#include "tx_batch_internal.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

namespace tx {

cudaError_t upload_batch_tables(const uint32_t lut[4][256][2]) {
    cudaError_t e = upload_tables_this_tu(lut);  // this unit's lane kernel
    if (e == cudaSuccess) e = upload_stage_tables<1>(lut);
    if (e == cudaSuccess) e = upload_stage_tables<2>(lut);
    if (e == cudaSuccess) e = upload_stage_tables<3>(lut);
    return e;
}

__global__ void __launch_bounds__(128, 5) k_batch_lanes(BatchQueue q) {
    __shared__ float s_unorm[256];
    __shared__ float s_sqrt[17];
    __shared__ float4 s_pts[16 * 128];
    init_unorm_tables(s_unorm, s_sqrt);
    const PointCol pt{s_pts + threadIdx.x, 128};
    const int lane = threadIdx.x & 31;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(q.counter, 1u);
        u = __shfl_sync(0xFFFFFFFFu, u, 0);
        if (u >= q.nunits) break;
        const uint2 unit = q.units[u];
        const BatchItem &it = q.items[unit.x];
        const SrcDesc src = it.src;
        const DevParams prm = it.prm;
        uint8_t *dst = it.dst;
        const int kind = it.kind, fmt = it.format, ch = it.channels;
        for (uint32_t k = 0; k < q.per_unit; ++k) {
            const uint32_t b = unit.y + 32u * k + (uint32_t)lane;
            if (b >= it.nblocks) break;
            if (kind == KIND_RANGE) {
                if (fmt == BC1) range_block<BC1>(src, b, prm, dst, s_unorm, s_sqrt, pt);
                else if (fmt == BC2) range_block<BC2>(src, b, prm, dst, s_unorm, s_sqrt, pt);
                else range_block<BC3>(src, b, prm, dst, s_unorm, s_sqrt, pt);
            } else if (fmt == BC4) {
                if (ch == 1) alpha_block<BC4, 1>(src, b, dst);
                else alpha_block<BC4, 4>(src, b, dst);
            } else {
                if (ch == 2) alpha_block<BC5, 2>(src, b, dst);
                else alpha_block<BC5, 4>(src, b, dst);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// mip producer: 2x2 box filter, (a+b+c+d+2)>>2 per channel, source
// coordinates clamped at odd edges.  (The reference builds no mips,
// cli/src/main.rs:153; this filter is the project's own definition.)

struct MipJobDev {
    const uint8_t *src;
    uint8_t *dst;
    uint32_t sw, sh, dw, dh;
    uint32_t spitch, dpitch;
    int32_t channels;
};

constexpr int kMipJobsPerLaunch = 256;  // 256 x 40 B of kernel parameters
struct MipJobs {
    MipJobDev job[kMipJobsPerLaunch];
};

__global__ void __launch_bounds__(256) k_mip(const __grid_constant__ MipJobs jobs, uint32_t njobs) {
    const uint32_t j = blockIdx.y;
    if (j >= njobs) return;
    const MipJobDev job = jobs.job[j];
    const uint32_t n = job.dw * job.dh;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t x = i % job.dw, y = i / job.dw;
        const uint32_t x0 = min(2 * x, job.sw - 1), x1 = min(2 * x + 1, job.sw - 1);
        const uint32_t y0 = min(2 * y, job.sh - 1), y1 = min(2 * y + 1, job.sh - 1);
        const uint8_t *r0 = job.src + (size_t)y0 * job.spitch, *r1 = job.src + (size_t)y1 * job.spitch;
        uint8_t *d = job.dst + (size_t)y * job.dpitch + (size_t)x * job.channels;
        for (int c = 0; c < job.channels; ++c) {
            const uint32_t s = r0[x0 * job.channels + c] + r0[x1 * job.channels + c] + r1[x0 * job.channels + c] +
                               r1[x1 * job.channels + c];
            d[c] = (uint8_t)((s + 2) >> 2);
        }
    }
}

}  // namespace tx

// ===========================================================================
// C ABI

struct tx_batch {
    int device = 0;
    std::vector<tx_batch_item> items;
    std::vector<tx::BatchItem> desc;
    tx::BatchItem *d_items = nullptr;
    uint2 *d_lane_units = nullptr, *d_team_units = nullptr;
    uint32_t *d_counters = nullptr;  // lane queue, then one per team class
    uint32_t n_lane = 0, n_team = 0;
    uint32_t team_counts[tx::kTeamClasses] = {};
    size_t nblocks = 0;
    tx_batch_tuning tuning{};
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    int sm_count = 0;
};

namespace {

constexpr int kTeamMaxThreads = 256;  // __launch_bounds__ of the k_batch_teams kernels

void default_tuning(tx_batch_tuning *t) {
    t->team_lanes = 32;
    t->team_threads_per_cta = 256;
    t->team_ctas_per_sm = 4;
    t->team_blocks_per_unit = 1;
    t->lane_ctas_per_sm = 3;
    t->lane_blocks_per_lane = 2;
    t->team_blocks_in_flight = 2;
}

void fill_tuning(const tx_batch_tuning *in, tx_batch_tuning *out) {
    default_tuning(out);
    if (!in) return;
    if (in->team_lanes == 16 || in->team_lanes == 32) out->team_lanes = in->team_lanes;
    if (in->team_threads_per_cta >= 64 && in->team_threads_per_cta <= kTeamMaxThreads &&
        in->team_threads_per_cta % 32 == 0)
        out->team_threads_per_cta = in->team_threads_per_cta;
    if (in->team_ctas_per_sm >= 1 && in->team_ctas_per_sm <= 16) out->team_ctas_per_sm = in->team_ctas_per_sm;
    if (in->team_blocks_per_unit >= 1 && in->team_blocks_per_unit <= 64) out->team_blocks_per_unit = in->team_blocks_per_unit;
    if (in->lane_ctas_per_sm >= 1 && in->lane_ctas_per_sm <= 16) out->lane_ctas_per_sm = in->lane_ctas_per_sm;
    if (in->lane_blocks_per_lane >= 1 && in->lane_blocks_per_lane <= 64) out->lane_blocks_per_lane = in->lane_blocks_per_lane;
    if (in->team_blocks_in_flight >= 1 && in->team_blocks_in_flight <= 3)
        out->team_blocks_in_flight = in->team_blocks_in_flight;
}

int fail_batch(cudaError_t e) {
    tx_internal_set_last_cuda_error((int)e);
    return e == cudaErrorMemoryAllocation ? TX_ERR_OUT_OF_MEMORY : TX_ERR_CUDA;
}

// (Re)build the unit queues for the current tuning and upload them.
int build_units(tx_batch *b) {
    std::vector<uint2> lane, cls[tx::kTeamClasses], team;
    const uint32_t lane_span = 32u * (uint32_t)b->tuning.lane_blocks_per_lane;
    const uint32_t team_span = (uint32_t)b->tuning.team_blocks_per_unit;
    for (uint32_t i = 0; i < b->desc.size(); ++i) {
        const tx::BatchItem &d = b->desc[i];
        if (d.kind == tx::KIND_ALPHA || d.kind == tx::KIND_RANGE) {
            for (uint32_t f = 0; f < d.nblocks; f += lane_span) lane.push_back(make_uint2(i, f));
        } else {
            auto &dst = cls[tx::team_class(d.format, d.kind)];
            for (uint32_t f = 0; f < d.nblocks; f += team_span) dst.push_back(make_uint2(i, f));
        }
    }
    for (int c = 0; c < tx::kTeamClasses; ++c) {  // class order: iterative (most expensive) first
        b->team_counts[c] = (uint32_t)cls[c].size();
        team.insert(team.end(), cls[c].begin(), cls[c].end());
    }
    cudaFree(b->d_lane_units);
    cudaFree(b->d_team_units);
    b->d_lane_units = b->d_team_units = nullptr;
    b->n_lane = (uint32_t)lane.size();
    b->n_team = (uint32_t)team.size();
    cudaError_t e;
    if (b->n_lane) {
        if ((e = cudaMalloc(&b->d_lane_units, lane.size() * sizeof(uint2))) != cudaSuccess) return fail_batch(e);
        if ((e = cudaMemcpy(b->d_lane_units, lane.data(), lane.size() * sizeof(uint2), cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail_batch(e);
    }
    if (b->n_team) {
        if ((e = cudaMalloc(&b->d_team_units, team.size() * sizeof(uint2))) != cudaSuccess) return fail_batch(e);
        if ((e = cudaMemcpy(b->d_team_units, team.data(), team.size() * sizeof(uint2), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return fail_batch(e);
    }
    return TX_OK;
}

cudaError_t launch_lanes(tx_batch *b, cudaStream_t st) {
    uint32_t grid = (uint32_t)(b->sm_count * b->tuning.lane_ctas_per_sm);
    const uint32_t need = (b->n_lane + 3) / 4;  // 4 warps per CTA
    if (grid > need) grid = need;
    if (grid == 0) grid = 1;
    tx::BatchQueue q{b->d_items, b->d_lane_units, b->n_lane, b->d_counters,
                     (uint32_t)b->tuning.lane_blocks_per_lane};
    tx::k_batch_lanes<<<grid, 128, 0, st>>>(q);
    tx::note_launch();
    return cudaGetLastError();
}

int launch_impl(tx_batch *b, cudaStream_t st) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(b->d_counters, 0, tx::kBatchCounters * sizeof(uint32_t), st)) != cudaSuccess)
        return fail_batch(e);
    const bool both = b->n_lane && b->n_team;
    if (both) {
        if ((e = cudaEventRecord(b->fork, st)) != cudaSuccess) return fail_batch(e);
        if ((e = cudaStreamWaitEvent(b->side, b->fork, 0)) != cudaSuccess) return fail_batch(e);
    }
    if (b->n_team) {
        e = tx::launch_team_classes(b->d_items, b->d_team_units, b->team_counts,
                                    (uint32_t)b->tuning.team_blocks_per_unit, b->d_counters + 1, b->sm_count,
                                    b->tuning, st);
        if (e != cudaSuccess) return fail_batch(e);
    }
    if (b->n_lane) {
        if ((e = launch_lanes(b, both ? b->side : st)) != cudaSuccess) return fail_batch(e);
    }
    if (both) {
        if ((e = cudaEventRecord(b->join, b->side)) != cudaSuccess) return fail_batch(e);
        if ((e = cudaStreamWaitEvent(st, b->join, 0)) != cudaSuccess) return fail_batch(e);
    }
    return TX_OK;
}

}  // namespace

extern "C" {

uint32_t tx_mip_count(uint32_t width, uint32_t height) {
    if (width == 0 || height == 0) return 0;
    uint32_t n = 1;
    while (width > 1 || height > 1) {
        width = width > 1 ? width >> 1 : 1;
        height = height > 1 ? height >> 1 : 1;
        ++n;
    }
    return n;
}

int tx_mip_batch_device(const tx_mip_job *jobs, size_t njobs, void *stream) {
    if (njobs == 0) return TX_OK;
    if (!jobs) return TX_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < njobs; ++i) {
        const tx_mip_job &j = jobs[i];
        if (!j.src || !j.dst || j.width == 0 || j.height == 0) return TX_ERR_INVALID_ARGUMENT;
        if (j.channels < 1 || j.channels > 4) return TX_ERR_INVALID_ARGUMENT;
        const uint32_t dw = j.width > 1 ? j.width >> 1 : 1;
        if (j.src_pitch < (size_t)j.width * j.channels || j.dst_pitch < (size_t)dw * j.channels)
            return TX_ERR_INVALID_ARGUMENT;
        if (j.src_pitch > 0xFFFFFFFFu || j.dst_pitch > 0xFFFFFFFFu) return TX_ERR_INVALID_ARGUMENT;
    }
    int rc = tx_internal_ensure_device();
    if (rc != TX_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // jobs travel as kernel parameters: no allocation, no copy, capturable
    for (size_t base = 0; base < njobs; base += tx::kMipJobsPerLaunch) {
        const size_t n = std::min<size_t>(tx::kMipJobsPerLaunch, njobs - base);
        tx::MipJobs pj;
        std::memset(&pj, 0, sizeof(pj));
        uint32_t maxpix = 0;
        for (size_t i = 0; i < n; ++i) {
            const tx_mip_job &j = jobs[base + i];
            const uint32_t dw = j.width > 1 ? j.width >> 1 : 1, dh = j.height > 1 ? j.height >> 1 : 1;
            pj.job[i] = tx::MipJobDev{static_cast<const uint8_t *>(j.src), static_cast<uint8_t *>(j.dst), j.width,
                                      j.height, dw, dh, (uint32_t)j.src_pitch, (uint32_t)j.dst_pitch, j.channels};
            maxpix = std::max(maxpix, dw * dh);
        }
        const uint32_t gx = std::min<uint32_t>((maxpix + 255) / 256, 1024);
        tx::k_mip<<<dim3(gx, (unsigned)n), 256, 0, st>>>(pj, (uint32_t)n);
        tx::note_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail_batch(e);
    }
    return TX_OK;
}

void tx_batch_default_tuning(tx_batch_tuning *t) {
    if (t) default_tuning(t);
}

int tx_batch_create(const tx_batch_item *items, size_t nitems, const tx_batch_tuning *tuning, tx_batch **out) {
    if (!out) return TX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (nitems && !items) return TX_ERR_INVALID_ARGUMENT;
    if (nitems > 0xFFFFFFFFu) return TX_ERR_INVALID_ARGUMENT;
    // argument checks first (host only), then the device
    for (size_t i = 0; i < nitems; ++i) {
        const tx_batch_item &it = items[i];
        const size_t bs = tx_block_size(it.format);
        const bool ch_ok = it.channels == 4 || (it.channels == 1 && it.format == TX_FORMAT_BC4) ||
                           (it.channels == 2 && it.format == TX_FORMAT_BC5);
        const int alg = it.params.algorithm;
        if (bs == 0) return TX_ERR_INVALID_FORMAT;
        if (!ch_ok || alg < TX_RANGE_FIT || alg > TX_ITERATIVE_CLUSTER_FIT || it.width == 0 ||
            it.src_pitch < (size_t)it.width * it.channels || (it.height && !it.src) || !it.dst)
            return TX_ERR_INVALID_ARGUMENT;
        if ((reinterpret_cast<uintptr_t>(it.dst) % bs) != 0) return TX_ERR_MISALIGNED;
        if (tx_num_blocks(it.width) * tx_num_blocks(it.height) > tx::kMaxBatchLevelBlocks)
            return TX_ERR_INVALID_ARGUMENT;
    }
    int rc = tx_internal_ensure_device();
    if (rc != TX_OK) return rc;
    tx_batch *b = new (std::nothrow) tx_batch();
    if (!b) return TX_ERR_OUT_OF_MEMORY;
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
    fill_tuning(tuning, &b->tuning);
    b->items.assign(items, items + nitems);
    b->desc.resize(nitems);
    for (size_t i = 0; i < nitems; ++i) {
        const tx_batch_item &it = items[i];
        tx::BatchItem &d = b->desc[i];
        std::memset(&d, 0, sizeof(d));
        const int f = it.format;
        const int alg = it.params.algorithm;
        const size_t nb = tx_num_blocks(it.width) * tx_num_blocks(it.height);
        d.src.base = static_cast<const uint8_t *>(it.src);
        d.src.masks = nullptr;
        d.src.pitch = it.src_pitch;
        d.src.width = it.width;
        d.src.height = it.height;
        tx::set_blocks_wide(d.src, (uint32_t)tx_num_blocks(it.width));
        d.src.channels = it.channels;
        const size_t va = it.channels == 4 ? 16 : (size_t)it.channels * 4;
        d.src.vec16 = ((reinterpret_cast<uintptr_t>(it.src) % va) == 0 && (it.src_pitch % va) == 0) ? 1 : 0;
        d.src.mode = 0;
        for (int c = 0; c < 3; ++c) d.prm.w[c] = it.params.weights[c];
        d.prm.alpha_weighted = it.params.weigh_colour_by_alpha ? 1 : 0;
        d.dst = static_cast<uint8_t *>(it.dst);
        d.nblocks = (uint32_t)nb;
        d.format = f;
        d.channels = it.channels;
        if (f == TX_FORMAT_BC4 || f == TX_FORMAT_BC5) d.kind = tx::KIND_ALPHA;
        else if (alg == TX_RANGE_FIT) d.kind = tx::KIND_RANGE;
        else d.kind = alg == TX_ITERATIVE_CLUSTER_FIT ? tx::KIND_CLUSTER_ITER : tx::KIND_CLUSTER;
        b->nblocks += nb;
    }
    cudaError_t e;
    if (nitems) {
        if ((e = cudaMalloc(&b->d_items, nitems * sizeof(tx::BatchItem))) != cudaSuccess) { tx_batch_destroy(b); return fail_batch(e); }
        if ((e = cudaMemcpy(b->d_items, b->desc.data(), nitems * sizeof(tx::BatchItem), cudaMemcpyHostToDevice)) != cudaSuccess) {
            tx_batch_destroy(b);
            return fail_batch(e);
        }
    }
    if ((e = cudaMalloc(&b->d_counters, tx::kBatchCounters * sizeof(uint32_t))) != cudaSuccess) {
        tx_batch_destroy(b);
        return fail_batch(e);
    }
    if ((e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming)) != cudaSuccess) {
        tx_batch_destroy(b);
        return fail_batch(e);
    }
    if ((rc = build_units(b)) != TX_OK) { tx_batch_destroy(b); return rc; }
    *out = b;
    return TX_OK;
}

int tx_batch_launch(tx_batch *b, void *stream) {
    if (!b) return TX_ERR_INVALID_ARGUMENT;
    nvtxRangePushA("tx_batch_launch");
    const int rc = launch_impl(b, static_cast<cudaStream_t>(stream));
    nvtxRangePop();
    return rc;
}

int tx_batch_set_tuning(tx_batch *b, const tx_batch_tuning *tuning) {
    if (!b || !tuning) return TX_ERR_INVALID_ARGUMENT;
    tx_batch_tuning t;
    fill_tuning(tuning, &t);
    const bool rebuild = t.team_blocks_per_unit != b->tuning.team_blocks_per_unit ||
                         t.lane_blocks_per_lane != b->tuning.lane_blocks_per_lane;
    b->tuning = t;
    return rebuild ? build_units(b) : TX_OK;
}

int tx_batch_get_tuning(const tx_batch *b, tx_batch_tuning *tuning) {
    if (!b || !tuning) return TX_ERR_INVALID_ARGUMENT;
    *tuning = b->tuning;
    return TX_OK;
}

int tx_batch_info(const tx_batch *b, size_t *nblocks, size_t *lane_units, size_t *team_units) {
    if (!b) return TX_ERR_INVALID_ARGUMENT;
    if (nblocks) *nblocks = b->nblocks;
    if (lane_units) *lane_units = b->n_lane;
    if (team_units) *team_units = b->n_team;
    return TX_OK;
}

// Project-written autotuner: coordinate descent over the launch shape, each
// candidate timed with CUDA events over `repeats` launches of this batch.
int tx_batch_autotune(tx_batch *b, void *stream, int repeats, tx_batch_tuning *chosen) {
    if (!b) return TX_ERR_INVALID_ARGUMENT;
    if (repeats < 1) repeats = 1;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    cudaError_t e;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess) return fail_batch(e);
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) { cudaEventDestroy(e0); return fail_batch(e); }
    int rc = TX_OK;
    auto measure = [&](const tx_batch_tuning &t, float *ms) -> int {
        int r = tx_batch_set_tuning(b, &t);
        if (r != TX_OK) return r;
        if ((r = launch_impl(b, st)) != TX_OK) return r;  // warm
        cudaEventRecord(e0, st);
        for (int i = 0; i < repeats; ++i)
            if ((r = launch_impl(b, st)) != TX_OK) return r;
        cudaEventRecord(e1, st);
        cudaError_t ee = cudaEventSynchronize(e1);
        if (ee != cudaSuccess) return fail_batch(ee);
        cudaEventElapsedTime(ms, e0, e1);
        return TX_OK;
    };
    tx_batch_tuning best = b->tuning;
    float best_ms = 0;
    if ((rc = measure(best, &best_ms)) == TX_OK) {
        struct Axis {
            int32_t tx_batch_tuning::*field;
            int opts[6];
            int n;
            bool team;
        };
        const Axis axes[] = {
            {&tx_batch_tuning::team_lanes, {32, 16}, 2, true},
            {&tx_batch_tuning::team_threads_per_cta, {64, 128, 256}, 3, true},
            {&tx_batch_tuning::team_ctas_per_sm, {1, 2, 3, 4, 6, 8}, 6, true},
            {&tx_batch_tuning::team_blocks_per_unit, {1, 2, 4, 8}, 4, true},
            {&tx_batch_tuning::team_blocks_in_flight, {1, 2, 3}, 3, true},
            {&tx_batch_tuning::lane_ctas_per_sm, {2, 3, 4, 6}, 4, false},
            {&tx_batch_tuning::lane_blocks_per_lane, {1, 2, 4, 8}, 4, false},
        };
        for (int pass = 0; pass < 2 && rc == TX_OK; ++pass) {
            for (const Axis &ax : axes) {
                if ((ax.team && !b->n_team) || (!ax.team && !b->n_lane)) continue;
                for (int i = 0; i < ax.n && rc == TX_OK; ++i) {
                    tx_batch_tuning t = best;
                    if (t.*ax.field == ax.opts[i]) continue;
                    t.*ax.field = ax.opts[i];
                    float ms = 0;
                    rc = measure(t, &ms);
                    if (rc == TX_OK && ms < best_ms) { best_ms = ms; best = t; }
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != TX_OK) return rc;
    rc = tx_batch_set_tuning(b, &best);
    if (chosen) *chosen = best;
    return rc;
}

void tx_batch_destroy(tx_batch *b) {
    if (!b) return;
    cudaFree(b->d_items);
    cudaFree(b->d_lane_units);
    cudaFree(b->d_team_units);
    cudaFree(b->d_counters);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    delete b;
}

}  // extern "C"

// ===========================================================================
// Allocation-free variant of the batch launch.
//
// Some callers cannot let a library call cudaMalloc: engines that reserve the
// whole device memory budget up front and hand out memory only through their
// own allocator, and per-frame loops that cannot afford the implicit device
// synchronisation an allocation or free may cause.  For them
// tx_batch_launch_noalloc compresses up to kNoallocMaxItems texture levels
// with the persistent batch kernels above, keeping the work queue (two
// counters, the item table, the units) in one file-scope device array of
// fixed size instead of memory from cudaMalloc.  Every GPU that loads this
// library holds the array until the process exits.  All calls share it and
// it keeps the last call's contents, so the set-up kernel clears the counters
// at the start of every call, and calls whose work overlaps on the GPU (two
// streams, or two host threads) race on it.

namespace tx {

constexpr size_t kNoallocScratchBytes = (size_t)1 << 20;  // 1 MiB per device
constexpr uint32_t kNoallocMaxItems = 256;                // texture levels per call
constexpr size_t kNoallocItemsOff = 256;                  // after the queue counters
constexpr size_t kNoallocUnitsOff =
    (kNoallocItemsOff + kNoallocMaxItems * sizeof(BatchItem) + 255) & ~(size_t)255;
constexpr uint32_t kNoallocMaxUnits = (uint32_t)((kNoallocScratchBytes - kNoallocUnitsOff) / sizeof(uint2));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

struct NoallocSetup {
    BatchItem items[kNoallocMaxItems];
    uint32_t nitems;
    uint32_t lane_span;  // blocks per lane unit (a multiple of 32)
    uint32_t team_span;  // blocks per team unit
};

// One CTA: copy the item table into the scratch array, clear the counters and
// write both unit queues (lane units first, then team units in item order,
// which the host has grouped by team class).
__global__ void __launch_bounds__(kNoallocMaxItems) k_noalloc_setup(const __grid_constant__ NoallocSetup p) {
    uint32_t *counters = reinterpret_cast<uint32_t *>(g_noalloc_scratch);
    BatchItem *items = reinterpret_cast<BatchItem *>(g_noalloc_scratch + kNoallocItemsOff);
    uint2 *units = reinterpret_cast<uint2 *>(g_noalloc_scratch + kNoallocUnitsOff);
    __shared__ uint32_t sl[kNoallocMaxItems], stm[kNoallocMaxItems];
    const uint32_t t = threadIdx.x;
    if (t < (uint32_t)kBatchCounters) counters[t] = 0;
    uint32_t nl = 0, nt = 0;
    if (t < p.nitems) {
        const BatchItem &it = p.items[t];
        items[t] = it;
        // 64-bit: nblocks < 2^31, but nblocks + span - 1 need not fit 32 bits
        if (it.kind == KIND_ALPHA || it.kind == KIND_RANGE)
            nl = (uint32_t)(((uint64_t)it.nblocks + p.lane_span - 1) / p.lane_span);
        else
            nt = (uint32_t)(((uint64_t)it.nblocks + p.team_span - 1) / p.team_span);
    }
    sl[t] = nl;
    stm[t] = nt;
    __syncthreads();
    for (uint32_t off = 1; off < kNoallocMaxItems; off <<= 1) {
        const uint32_t a = t >= off ? sl[t - off] : 0u, b = t >= off ? stm[t - off] : 0u;
        __syncthreads();
        sl[t] += a;
        stm[t] += b;
        __syncthreads();
    }
    const uint32_t lane_base = sl[t] - nl;
    const uint32_t team_base = sl[kNoallocMaxItems - 1] + stm[t] - nt;
    for (uint32_t k = 0; k < nl; ++k) units[lane_base + k] = make_uint2(t, k * p.lane_span);
    for (uint32_t k = 0; k < nt; ++k) units[team_base + k] = make_uint2(t, k * p.team_span);
}

}  // namespace tx

namespace {

struct NoallocDevice {
    bool ready = false;
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
    int sm_count = 0;
};
NoallocDevice g_noalloc_dev[64];
std::mutex g_noalloc_mu;

// Per-device set-up, done by the first call on each device (with that device
// current): the device address of the scratch array, the SM count and the
// team kernel's shared-memory limit.
int noalloc_setup_device(int dev, NoallocDevice **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocDevice &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, tx::g_noalloc_scratch);
        if (e != cudaSuccess) return fail_batch(e);
        if ((e = cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return fail_batch(e);
        if ((e = tx::prepare_team_kernels()) != cudaSuccess) return fail_batch(e);
        d.scratch = static_cast<unsigned char *>(ptr);
        d.ready = true;
    }
    *out = &d;
    return TX_OK;
}

}  // namespace

extern "C" int tx_batch_launch_noalloc(const tx_batch_item *items, size_t nitems, void *stream) {
    if (nitems == 0) return TX_OK;
    if (!items || nitems > tx::kNoallocMaxItems) return TX_ERR_INVALID_ARGUMENT;
    static_assert(sizeof(tx::NoallocSetup) <= 32000, "kernel parameter block too large");
    tx::NoallocSetup setup;
    std::memset(&setup, 0, sizeof(setup));
    // order: lane items first, then the ClusterFit items by team class
    // (iterative first), so the team queue comes out grouped by class
    uint32_t n = 0;
    for (int pass = 0; pass <= tx::kTeamClasses; ++pass) {
        for (size_t i = 0; i < nitems; ++i) {
            const tx_batch_item &it = items[i];
            const size_t bs = tx_block_size(it.format);
            const bool ch_ok = it.channels == 4 || (it.channels == 1 && it.format == TX_FORMAT_BC4) ||
                               (it.channels == 2 && it.format == TX_FORMAT_BC5);
            const int alg = it.params.algorithm;
            if (bs == 0) return TX_ERR_INVALID_FORMAT;
            if (!ch_ok || alg < TX_RANGE_FIT || alg > TX_ITERATIVE_CLUSTER_FIT || it.width == 0 ||
                it.src_pitch < (size_t)it.width * it.channels || (it.height && !it.src) || !it.dst)
                return TX_ERR_INVALID_ARGUMENT;
            if ((reinterpret_cast<uintptr_t>(it.dst) % bs) != 0) return TX_ERR_MISALIGNED;
            const size_t nb = tx_num_blocks(it.width) * tx_num_blocks(it.height);
            if (nb > tx::kMaxBatchLevelBlocks) return TX_ERR_INVALID_ARGUMENT;
            const bool lane = it.format == TX_FORMAT_BC4 || it.format == TX_FORMAT_BC5 || alg == TX_RANGE_FIT;
            const int kind = lane ? (alg == TX_RANGE_FIT && it.format <= TX_FORMAT_BC3 ? tx::KIND_RANGE : tx::KIND_ALPHA)
                                  : (alg == TX_ITERATIVE_CLUSTER_FIT ? tx::KIND_CLUSTER_ITER : tx::KIND_CLUSTER);
            if (pass != (lane ? 0 : 1 + tx::team_class(it.format, kind))) continue;
            tx::BatchItem &d = setup.items[n++];
            d.src.base = static_cast<const uint8_t *>(it.src);
            d.src.masks = nullptr;
            d.src.pitch = it.src_pitch;
            d.src.width = it.width;
            d.src.height = it.height;
            tx::set_blocks_wide(d.src, (uint32_t)tx_num_blocks(it.width));
            d.src.channels = it.channels;
            const size_t va = it.channels == 4 ? 16 : (size_t)it.channels * 4;
            d.src.vec16 = ((reinterpret_cast<uintptr_t>(it.src) % va) == 0 && (it.src_pitch % va) == 0) ? 1 : 0;
            d.src.mode = 0;
            for (int c = 0; c < 3; ++c) d.prm.w[c] = it.params.weights[c];
            d.prm.alpha_weighted = it.params.weigh_colour_by_alpha ? 1 : 0;
            d.dst = static_cast<uint8_t *>(it.dst);
            d.nblocks = (uint32_t)nb;
            d.format = it.format;
            d.channels = it.channels;
            d.kind = kind;
        }
    }
    setup.nitems = n;
    // unit sizes: the defaults, doubled until both queues fit the scratch array
    uint32_t lane_span = 64, team_span = 1;
    uint32_t team_counts[tx::kTeamClasses] = {};
    auto count_units = [&](uint64_t *nl, uint64_t *nt) {
        *nl = *nt = 0;
        for (int c = 0; c < tx::kTeamClasses; ++c) team_counts[c] = 0;
        for (uint32_t i = 0; i < n; ++i) {
            const tx::BatchItem &d = setup.items[i];
            if (d.kind == tx::KIND_ALPHA || d.kind == tx::KIND_RANGE) {
                *nl += ((uint64_t)d.nblocks + lane_span - 1) / lane_span;
            } else {
                const uint32_t u = (uint32_t)(((uint64_t)d.nblocks + team_span - 1) / team_span);
                *nt += u;
                team_counts[tx::team_class(d.format, d.kind)] += u;
            }
        }
    };
    uint64_t n_lane = 0, n_team = 0;
    count_units(&n_lane, &n_team);
    while (n_lane + n_team > tx::kNoallocMaxUnits) {
        if (n_team >= n_lane) team_span *= 2;
        else lane_span *= 2;
        count_units(&n_lane, &n_team);
    }
    setup.lane_span = lane_span;
    setup.team_span = team_span;

    int rc = tx_internal_ensure_device();
    if (rc != TX_OK) return rc;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_batch(e);
    if (dev < 0 || dev >= 64) return TX_ERR_NO_DEVICE;
    NoallocDevice *nd = nullptr;
    if ((rc = noalloc_setup_device(dev, &nd)) != TX_OK) return rc;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const tx::BatchItem *d_items = reinterpret_cast<const tx::BatchItem *>(nd->scratch + tx::kNoallocItemsOff);
    const uint2 *d_units = reinterpret_cast<const uint2 *>(nd->scratch + tx::kNoallocUnitsOff);
    uint32_t *d_counters = reinterpret_cast<uint32_t *>(nd->scratch);
    tx::k_noalloc_setup<<<1, tx::kNoallocMaxItems, 0, st>>>(setup);
    tx::note_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_batch(e);
    if (n_lane) {
        tx::BatchQueue q{d_items, d_units, (uint32_t)n_lane, d_counters, lane_span / 32};
        uint32_t grid = (uint32_t)(nd->sm_count * 3);
        grid = std::min<uint32_t>(grid, (uint32_t)((n_lane + 3) / 4));
        tx::k_batch_lanes<<<grid, 128, 0, st>>>(q);
        tx::note_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return fail_batch(e);
    }
    if (n_team) {
        tx_batch_tuning t;
        default_tuning(&t);
        if ((e = tx::launch_team_classes(d_items, d_units + n_lane, team_counts, team_span, d_counters + 1,
                                         nd->sm_count, t, st)) != cudaSuccess)
            return fail_batch(e);
    }
    return TX_OK;
}

// ===========================================================================
// helpers for the serving loop (tx_server.cu)

namespace tx {

void fill_batch_item(const tx_batch_item &it, BatchItem *d) {
    std::memset(d, 0, sizeof(*d));
    d->src.base = static_cast<const uint8_t *>(it.src);
    d->src.pitch = it.src_pitch;
    d->src.width = it.width;
    d->src.height = it.height;
    tx::set_blocks_wide(d->src, (uint32_t)tx_num_blocks(it.width));
    d->src.channels = it.channels;
    const size_t va = it.channels == 4 ? 16 : (size_t)it.channels * 4;
    d->src.vec16 = ((reinterpret_cast<uintptr_t>(it.src) % va) == 0 && (it.src_pitch % va) == 0) ? 1 : 0;
    for (int c = 0; c < 3; ++c) d->prm.w[c] = it.params.weights[c];
    d->prm.alpha_weighted = it.params.weigh_colour_by_alpha ? 1 : 0;
    d->dst = static_cast<uint8_t *>(it.dst);
    d->nblocks = (uint32_t)(tx_num_blocks(it.width) * tx_num_blocks(it.height));
    d->format = it.format;
    d->channels = it.channels;
    const int alg = it.params.algorithm;
    if (it.format == TX_FORMAT_BC4 || it.format == TX_FORMAT_BC5) d->kind = KIND_ALPHA;
    else if (alg == TX_RANGE_FIT) d->kind = KIND_RANGE;
    else d->kind = alg == TX_ITERATIVE_CLUSTER_FIT ? KIND_CLUSTER_ITER : KIND_CLUSTER;
}

cudaError_t prepare_team_kernels() {
    // the default staging depth, the one the allocation-free launch uses
    return prepare_team_class_kernels<2>();
}

cudaError_t launch_team_classes(const BatchItem *d_items, const uint2 *d_team,
                                const uint32_t (&team_counts)[kTeamClasses], uint32_t team_blocks_per_unit,
                                uint32_t *counters, int sm_count, const tx_batch_tuning &t, cudaStream_t st) {
    const int threads = t.team_threads_per_cta;
    const int team = t.team_lanes == 16 ? 16 : 32;
    const uint32_t per = (uint32_t)(threads / team);
    uint32_t begin = 0;
    for (int c = 0; c < kTeamClasses; ++c) {
        const uint32_t n = team_counts[c];
        if (n == 0) continue;
        uint32_t grid = (uint32_t)(sm_count * t.team_ctas_per_sm);
        grid = std::max<uint32_t>(1, std::min<uint32_t>(grid, (n + per - 1) / per));
        const BatchQueue q{d_items, d_team + begin, n, counters + c, team_blocks_per_unit};
        begin += n;
        const cudaError_t e = t.team_blocks_in_flight == 1   ? launch_team_class<1>(team, c, q, grid, threads, st)
                              : t.team_blocks_in_flight == 3 ? launch_team_class<3>(team, c, q, grid, threads, st)
                                                             : launch_team_class<2>(team, c, q, grid, threads, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_batch_queues(const BatchItem *d_items, const uint2 *d_lane, uint32_t n_lane,
                                uint32_t lane_blocks_per_lane, const uint2 *d_team,
                                const uint32_t (&team_counts)[kTeamClasses], uint32_t team_blocks_per_unit,
                                uint32_t *d_counters, int sm_count, const tx_batch_tuning &t, cudaStream_t st) {
    if (n_lane) {
        uint32_t grid = (uint32_t)(sm_count * t.lane_ctas_per_sm);
        grid = std::max<uint32_t>(1, std::min<uint32_t>(grid, (n_lane + 3) / 4));
        BatchQueue q{d_items, d_lane, n_lane, d_counters, lane_blocks_per_lane};
        k_batch_lanes<<<grid, 128, 0, st>>>(q);
        note_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_team_classes(d_items, d_team, team_counts, team_blocks_per_unit, d_counters + 1, sm_count, t, st);
}

}  // namespace tx
