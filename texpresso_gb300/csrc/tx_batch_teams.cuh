// tx_batch_teams.cuh -- the persistent ClusterFit team kernel of the batched
// and serving forms, with a staging depth: STAGE blocks whose pixels a team
// holds or has requested at any time (1 = load a block, then encode it; 2 =
// request the next block's pixels before encoding the current one; 3 = two
// blocks ahead).  Each depth is compiled in its own translation unit
// (tx_batch_stage1/2/3.cu), which also keeps the build parallel; the
// autotuner picks the depth (tx_batch_tuning.team_blocks_in_flight).
#pragma once
#include "tx_batch_internal.h"
#include "tx_colour.cuh"
#include "tx_internal.h"

namespace tx {

// One team class: every unit of q is (FMT, NITER).  Teams pop units (runs of
// blocks of one level) with one atomicAdd; the blocks of the current unit and
// then of the next units form a stream, of which the next STAGE blocks are
// staged (pixel requested, one per lane) while the oldest one is encoded.
template <int TEAM, int FMT, int NITER, int STAGE>
__global__ void __launch_bounds__(256, 4) k_batch_teams(BatchQueue q) {
    static_assert(STAGE >= 1 && STAGE <= 3, "staging depth");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float s_unorm[256];
    __shared__ float s_sqrt[17];
    init_unorm_tables(s_unorm, s_sqrt);
    TeamSmem *teams = reinterpret_cast<TeamSmem *>(smem_raw);
    const TeamTables tt{g_cand, g_cand + kCand4 + 1, s_unorm, s_sqrt};
    const Team<TEAM> tm;
    TeamSmem &sm = teams[threadIdx.x / TEAM];

    // cursor: the next block to stage (item ci, block cb of a unit ending at ce)
    uint32_t ci = 0, cb = 0, ce = 0;
    auto pop = [&]() {
        uint32_t u = 0;
        if (tm.lane == 0) u = atomicAdd(q.counter, 1u);
        u = tm.shfl(u, 0);
        if (u >= q.nunits) return false;
        const uint2 unit = q.units[u];
        ci = unit.x;
        cb = unit.y;
        // 64-bit: first block + blocks per unit need not fit 32 bits
        ce = (uint32_t)min((uint64_t)unit.y + q.per_unit, (uint64_t)q.items[unit.x].nblocks);
        return true;
    };
    auto next = [&]() { return ++cb < ce || pop(); };
    bool more = pop();

    // staged blocks, oldest first: item, block, this lane's pixel
    uint32_t si[STAGE], sb[STAGE];
    TeamPixel sp[STAGE];
    bool sok[STAGE];
#pragma unroll
    for (int s = 0; s < STAGE - 1; ++s) {  // fill all but the newest slot
        sok[s] = more;
        si[s] = ci;
        sb[s] = cb;
        sp[s] = more ? load_team_pixel(q.items[ci].src, cb, tm.lane) : TeamPixel{0u, false};
        if (more) more = next();
    }
    for (;;) {
        // request the newest block before encoding the oldest one
        sok[STAGE - 1] = more;
        si[STAGE - 1] = ci;
        sb[STAGE - 1] = cb;
        sp[STAGE - 1] = more ? load_team_pixel(q.items[ci].src, cb, tm.lane) : TeamPixel{0u, false};
        if (more) more = next();
        if (!sok[0]) break;
        const BatchItem &it = q.items[si[0]];
        cluster_block_px<FMT, TEAM, NITER>(tm, sm, tt, sp[0], sb[0], it.prm, it.dst);
#pragma unroll
        for (int s = 0; s < STAGE - 1; ++s) {
            sok[s] = sok[s + 1];
            si[s] = si[s + 1];
            sb[s] = sb[s + 1];
            sp[s] = sp[s + 1];
        }
    }
}

// The team kernels need more than 48 KB of dynamic shared memory: raise the
// limit once per device and kernel.
template <int TEAM, int FMT, int NITER, int STAGE>
static cudaError_t class_attr() {
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !attr_set[dev]) {
        const cudaError_t e = cudaFuncSetAttribute(k_batch_teams<TEAM, FMT, NITER, STAGE>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)cluster_smem_bytes(TEAM, 256));
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    return cudaSuccess;
}

template <int TEAM, int FMT, int NITER, int STAGE>
static cudaError_t launch_one_class(const BatchQueue &q, uint32_t grid, int threads, cudaStream_t st) {
    const cudaError_t e = class_attr<TEAM, FMT, NITER, STAGE>();
    if (e != cudaSuccess) return e;
    k_batch_teams<TEAM, FMT, NITER, STAGE><<<grid, threads, cluster_smem_bytes(TEAM, threads), st>>>(q);
    note_launch();
    return cudaGetLastError();
}

template <int TEAM, int STAGE>
static cudaError_t launch_class_t(int c, const BatchQueue &q, uint32_t grid, int threads, cudaStream_t st) {
    switch (c) {
    case 0: return launch_one_class<TEAM, BC1, 8, STAGE>(q, grid, threads, st);
    case 1: return launch_one_class<TEAM, BC2, 8, STAGE>(q, grid, threads, st);
    case 2: return launch_one_class<TEAM, BC3, 8, STAGE>(q, grid, threads, st);
    case 3: return launch_one_class<TEAM, BC1, 1, STAGE>(q, grid, threads, st);
    case 4: return launch_one_class<TEAM, BC2, 1, STAGE>(q, grid, threads, st);
    case 5: return launch_one_class<TEAM, BC3, 1, STAGE>(q, grid, threads, st);
    default: return cudaErrorInvalidValue;
    }
}

// Definitions of the per-depth entry points declared in tx_batch_internal.h;
// tx_batch_stage<N>.cu instantiates them for its N.
template <int STAGE>
cudaError_t launch_team_class(int team, int c, const BatchQueue &q, uint32_t grid, int threads, cudaStream_t st) {
    return team == 16 ? launch_class_t<16, STAGE>(c, q, grid, threads, st)
                      : launch_class_t<32, STAGE>(c, q, grid, threads, st);
}

template <int STAGE>
cudaError_t prepare_team_class_kernels() {
    cudaError_t e;
    if ((e = class_attr<32, BC1, 8, STAGE>()) != cudaSuccess || (e = class_attr<32, BC2, 8, STAGE>()) != cudaSuccess ||
        (e = class_attr<32, BC3, 8, STAGE>()) != cudaSuccess || (e = class_attr<32, BC1, 1, STAGE>()) != cudaSuccess ||
        (e = class_attr<32, BC2, 1, STAGE>()) != cudaSuccess || (e = class_attr<32, BC3, 1, STAGE>()) != cudaSuccess)
        return e;
    return cudaSuccess;
}

template <int STAGE>
cudaError_t upload_stage_tables(const uint32_t lut[4][256][2]) {
    return upload_tables_this_tu(lut);
}

}  // namespace tx
