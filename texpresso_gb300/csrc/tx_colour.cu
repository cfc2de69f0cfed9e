// tx_colour.cu -- single-texture BC1/BC2/BC3 kernels and their launchers
// (device code in tx_colour.cuh).
#include "tx_colour.cuh"
#include "tx_internal.h"

#include <cstdlib>

namespace tx {

template <int FMT>
__global__ void __launch_bounds__(128, 6) k_range(SrcDesc src, DevParams prm, uint8_t *__restrict__ out,
                                               size_t nblocks) {
    __shared__ float s_unorm[256];
    __shared__ float s_sqrt[17];
    __shared__ float4 s_pts[16 * 128];
    init_unorm_tables(s_unorm, s_sqrt);
    const PointCol pt{s_pts + threadIdx.x, 128};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t b = (size_t)blockIdx.x * blockDim.x + threadIdx.x; b < nblocks; b += stride)
        range_block<FMT>(src, b, prm, out, s_unorm, s_sqrt, pt);
}

template <int FMT, int TEAM, int NITER>
__global__ void __launch_bounds__(256, 4) k_cluster(SrcDesc src, DevParams prm, uint8_t *__restrict__ out,
                                                 size_t nblocks) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // The u8 -> [0,1] and sqrt(count) tables: a ClusterFit CTA (8 blocks, then
    // the next CTA) reads them from global memory through L1, because building
    // them in shared memory cost each CTA 256 divisions and a barrier (BC3
    // 2048x2048: 742 vs 776 us); the persistent IterativeClusterFit CTAs build
    // them once and read shared memory (991 vs 999 us).
    __shared__ float s_unorm[256];
    __shared__ float s_sqrt[17];
    __shared__ uint32_t s_next;
    if (NITER > 1) {
        if (threadIdx.x == 0) s_next = 0;
        init_unorm_tables(s_unorm, s_sqrt);  // ends with __syncthreads
    }
    TeamSmem *teams = reinterpret_cast<TeamSmem *>(smem_raw);
    const TeamTables tt{g_cand, g_cand + kCand4 + 1, NITER > 1 ? s_unorm : g_unorm8, NITER > 1 ? s_sqrt : g_sqrt_count};
    const Team<TEAM> tm;
    TeamSmem &sm = teams[threadIdx.x / TEAM];
    if (NITER == 1) {
        // ClusterFit: team t of CTA c encodes block c * teams + t (grid-strided)
        const int teams_per_cta = blockDim.x / TEAM;
        const size_t nteams = (size_t)gridDim.x * teams_per_cta;
        for (size_t b = (size_t)blockIdx.x * teams_per_cta + threadIdx.x / TEAM; b < nblocks; b += nteams)
            cluster_block<FMT, TEAM, NITER>(tm, sm, tt, src, b, prm, out);
        return;
    }
    // IterativeClusterFit (persistent CTAs): CTA c owns the chunks of 8
    // neighbouring blocks c, c + grid, c + 2 grid, ..., and its teams take the
    // blocks one at a time from a shared counter, so a team that drew cheap
    // blocks (one colour, one ordering) takes more of them instead of idling
    // until the CTA's slowest team is done, and teams working at the same time
    // still read neighbouring pixels.  For BC2/BC3 the next block's pixels are
    // requested before the current block is encoded; BC1, whose compress3 +
    // compress4 code already runs at the register limit, measured faster
    // without that (163 vs 159 Mblocks/s; BC3: 254 vs 265).
    auto take = [&]() {
        uint32_t k = 0;
        if (tm.lane == 0) k = atomicAdd(&s_next, 1u);
        k = tm.shfl(k, 0);
        return ((size_t)(k >> 3) * gridDim.x + blockIdx.x) * 8u + (k & 7u);
    };
    const size_t end_chunk = (nblocks + 7) / 8 * 8;  // slots past this belong to no chunk
    if (FMT == BC1) {
        for (size_t b = take(); b < end_chunk; b = take())
            if (b < nblocks) cluster_block_px<FMT, TEAM, NITER>(tm, sm, tt, load_team_pixel(src, b, tm.lane), b, prm, out);
        return;
    }
    size_t b = take();
    TeamPixel tp{0u, false};
    if (b < nblocks) tp = load_team_pixel(src, b, tm.lane);
    while (b < end_chunk) {
        const size_t bn = take();
        TeamPixel tn{0u, false};
        if (bn < nblocks) tn = load_team_pixel(src, bn, tm.lane);
        if (b < nblocks) cluster_block_px<FMT, TEAM, NITER>(tm, sm, tt, tp, b, prm, out);
        b = bn;
        tp = tn;
    }
}

size_t cluster_smem_bytes(int team, int threads) {
    return (size_t)(threads / team) * sizeof(TeamSmem);
}

cudaError_t upload_colour_tables(const uint32_t lut[4][256][2]) { return upload_tables_this_tu(lut); }

template <int FMT>
static cudaError_t launch_range_t(const SrcDesc &src, const DevParams &prm, uint8_t *out, size_t nblocks,
                                  cudaStream_t st, const LaunchCfg &cfg) {
    const int threads = 128;
    size_t grid = (nblocks + threads - 1) / threads;
    if (grid > cfg.max_ctas) grid = cfg.max_ctas;
    if (grid == 0) grid = 1;
    k_range<FMT><<<(unsigned)grid, threads, 0, st>>>(src, prm, out, nblocks);
    note_launch();
    return cudaGetLastError();
}

template <int FMT, int TEAM, int NITER>
static cudaError_t launch_cluster_t(const SrcDesc &src, const DevParams &prm, uint8_t *out, size_t nblocks,
                                    cudaStream_t st, const LaunchCfg &cfg) {
    // A launch smaller than one wave of 8-team CTAs (SMs x 4 x 8 blocks) runs
    // in one-warp CTAs: they spread evenly over the SMs (for 4,096 blocks, 26-28
    // on an SM against 3-4 CTAs of 8 teams), and a team that finishes frees
    // its slot without waiting for CTA partners; the slowest SM sets the
    // launch's time.  (256x256 BC1: 25.9 us in one-warp CTAs, 26.5 us in
    // 2-team and 26.9 us in 4-team CTAs.)
    static int sm_count[64] = {};
    int dev0 = 0;
    cudaGetDevice(&dev0);
    if (dev0 < 64 && sm_count[dev0] == 0) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev0) == cudaSuccess && sms > 0)
            sm_count[dev0] = sms;
    }
    int threads = cfg.cluster_threads;
    if (NITER == 1 && threads == 256 && dev0 < 64 && sm_count[dev0] > 0 &&
        nblocks < (size_t)sm_count[dev0] * 4 * (256 / TEAM))
        threads = 32;
    const size_t smem = cluster_smem_bytes(TEAM, threads);
    static bool attr_set[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_cluster<FMT, TEAM, NITER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)cluster_smem_bytes(TEAM, 256));
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    // IterativeClusterFit: one wave of persistent CTAs (SMs x resident CTAs),
    // whose teams deal blocks among themselves, because blocks needing 1 or 2+
    // orderings differ twofold in cost.  ClusterFit: one chunk per CTA (the
    // hardware schedules CTAs as slots free up, which measured faster there).
    static int resident[64] = {};
    if (NITER > 1 && dev < 64 && resident[dev] == 0) {
        int sms = 0, per_sm = 0;
        cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cluster<FMT, TEAM, NITER>, 256,
                                                              cluster_smem_bytes(TEAM, 256));
        if (e != cudaSuccess) return e;
        resident[dev] = sms * (per_sm > 0 ? per_sm : 1);
    }
    const size_t teams_per_cta = (size_t)threads / TEAM;
    size_t grid = NITER > 1 ? (nblocks + 7) / 8 : (nblocks + teams_per_cta - 1) / teams_per_cta;  // chunks : blocks
    if (NITER > 1) {
        const size_t wave = (size_t)(dev < 64 ? resident[dev] : 1) * (256 / threads);
        if (grid > wave) grid = wave;
    }
    if (grid > cfg.max_ctas) grid = cfg.max_ctas;
    if (grid == 0) grid = 1;
    k_cluster<FMT, TEAM, NITER><<<(unsigned)grid, threads, smem, st>>>(src, prm, out, nblocks);
    note_launch();
    return cudaGetLastError();
}

// Lanes per block of the single-texture ClusterFit kernel: 32 unless the
// TX_CLUSTER_TEAM environment variable asks for 16 (read once).
static int cluster_team_override() {
    static const int v = [] {
        const char *e = getenv("TX_CLUSTER_TEAM");
        return (e && atoi(e) == 16) ? 16 : (e && atoi(e) == 32) ? 32 : 0;
    }();
    return v;
}

template <int FMT, int NITER>
static cudaError_t launch_cluster_team(const SrcDesc &src, const DevParams &prm, uint8_t *out, size_t nblocks,
                                       cudaStream_t st, const LaunchCfg &cfg) {
    const int team = cluster_team_override() ? cluster_team_override() : cfg.cluster_team;
    if (team == 16) return launch_cluster_t<FMT, 16, NITER>(src, prm, out, nblocks, st, cfg);
    return launch_cluster_t<FMT, 32, NITER>(src, prm, out, nblocks, st, cfg);
}

cudaError_t launch_colour(int fmt, int algorithm, const SrcDesc &src, const DevParams &prm, uint8_t *out,
                          size_t nblocks, cudaStream_t st, const LaunchCfg &cfg) {
    if (nblocks == 0) return cudaSuccess;
    if (algorithm == RANGE_FIT) {
        switch (fmt) {
        case BC1: return launch_range_t<BC1>(src, prm, out, nblocks, st, cfg);
        case BC2: return launch_range_t<BC2>(src, prm, out, nblocks, st, cfg);
        case BC3: return launch_range_t<BC3>(src, prm, out, nblocks, st, cfg);
        default: return cudaErrorInvalidValue;
        }
    }
    const bool iter = algorithm == ITERATIVE_CLUSTER_FIT;
    switch (fmt) {
    case BC1: return iter ? launch_cluster_team<BC1, 8>(src, prm, out, nblocks, st, cfg)
                          : launch_cluster_team<BC1, 1>(src, prm, out, nblocks, st, cfg);
    case BC2: return iter ? launch_cluster_team<BC2, 8>(src, prm, out, nblocks, st, cfg)
                          : launch_cluster_team<BC2, 1>(src, prm, out, nblocks, st, cfg);
    case BC3: return iter ? launch_cluster_team<BC3, 8>(src, prm, out, nblocks, st, cfg)
                          : launch_cluster_team<BC3, 1>(src, prm, out, nblocks, st, cfg);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tx
