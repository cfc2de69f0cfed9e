// tx_server.cu -- serving form: a request loop with admission by free device
// memory and continuous batching.
//
// A server owns a stream-ordered memory pool, three streams (host->device
// copies and mip generation, compression steps, device->host copies) and one
// worker thread.  Requests are admitted first-in first-out while two limits
// allow: the bytes held by admitted requests stay within the budget, and the
// device's free memory right now (cudaMemGetInfo, plus what the pool holds
// but no request uses) covers the request with a fixed headroom left over for
// everything else on the device.  An admitted request gets its device memory
// from the pool on the copy stream; its pixels are copied in and its mip chain
// built there, overlapping the running compression steps.  Every step is one
// launch of the persistent batch kernels over a work queue assembled from all
// ready requests: each gets a round-robin share of blocks, so requests that
// arrive while others run join the very next step and small requests finish
// without waiting for large ones.  Two steps are kept in flight; the queue of
// step n+1 is written while step n runs.  When a request's last blocks have
// been compressed its levels are copied back on the third stream and its
// memory goes back to the pool behind those copies.
//
// Each block is encoded by the same per-block code as every other entry point,
// so a request's bytes do not depend on what else is in flight.  The loop is
// scheduled from the host: a step is a kernel launch, so no kernel waits on
// another or on the host.
#include "texpresso_gb300.h"
#include "tx_batch_internal.h"
#include "tx_internal.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

double now_us() {
    using namespace std::chrono;
    return (double)duration_cast<nanoseconds>(steady_clock::now().time_since_epoch()).count() * 1e-3;
}

constexpr size_t kAlign = 256;
size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

// Device memory left free for everything else on the device (other
// libraries' caches, other processes) when admitting a request.
constexpr size_t kHbmHeadroom = (size_t)1 << 30;

struct Level {
    uint32_t w, h, nblocks;
    size_t src_off, dst_off, dst_bytes, out_off;
};

struct Request {
    uint64_t id = 0;
    tx_server_request r{};
    std::vector<Level> levels;
    size_t footprint = 0;
    uint8_t *dev = nullptr;  // the request's device memory (from the server's pool)
    enum State { QUEUED, LOADING, ACTIVE, DRAINING, DONE } state = QUEUED;
    std::vector<uint32_t> next_block;
    size_t unassigned = 0;
    cudaEvent_t ready_ev = nullptr, done_ev = nullptr;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int status = TX_OK;
    uint32_t steps = 0;
    bool hbm_deferred = false;          // worker only: counted once in hbm_waits
    std::atomic<bool> finished{false};  // set under tx_server::mu; read by waiters
    bool cancel = false;                // guarded by tx_server::mu
    bool admitted = false;              // guarded by tx_server::mu
};

struct Step {
    tx::BatchItem *d_items = nullptr;
    uint2 *d_units = nullptr;
    uint32_t *d_counters = nullptr;
    tx::BatchItem *h_items = nullptr;  // pinned staging
    uint2 *h_units = nullptr;          // pinned staging
    cudaEvent_t start = nullptr, done = nullptr;  // timing: the step's time on the compression stream
    std::vector<Request *> finishing;
    bool busy = false;
};

}  // namespace

struct tx_server {
    tx_server_config cfg{};
    int device = 0, sm_count = 0;
    cudaMemPool_t pool = nullptr;
    size_t held = 0, held_high = 0;  // bytes held by admitted requests (worker only; stats under mu)
    double busy_us = 0;              // compression-step time on the device (worker only; stats under mu)
    uint64_t hbm_waits = 0;          // admissions deferred for lack of free device memory
    double hbm_retry_at = 0;         // worker only: earliest time to query free memory again
    cudaStream_t s_load = nullptr, s_comp = nullptr, s_store = nullptr;
    Step steps[2];
    uint32_t max_items = 0, max_units = 0;
    uint64_t step_count = 0;
    int next_step = 0;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> submitted;                   // guarded by mu
    std::unordered_map<uint64_t, Request *> requests;  // guarded by mu
    uint64_t next_id = 1;
    bool stopping = false;
    int fatal = TX_OK;
    uint64_t n_submitted = 0, n_completed = 0;

    std::deque<Request *> waiting;   // worker only: not yet admitted
    std::vector<Request *> live;     // worker only: admitted, not done
    size_t rr = 0;                   // round-robin cursor
    std::thread worker;
};

namespace {

int fail_server(cudaError_t e) {
    tx_internal_set_last_cuda_error((int)e);
    return e == cudaErrorMemoryAllocation ? TX_ERR_OUT_OF_MEMORY : TX_ERR_CUDA;
}

void plan_levels(Request *q) {
    const tx_server_request &r = q->r;
    uint32_t w = r.width, h = r.height;
    const uint32_t n = r.mips ? tx_mip_count(w, h) : 1;
    size_t off = 0, out = 0;
    for (uint32_t l = 0; l < n; ++l) {
        Level lv;
        lv.w = w;
        lv.h = h;
        lv.nblocks = (uint32_t)(tx_num_blocks(w) * tx_num_blocks(h));
        lv.src_off = off;
        off += align_up((size_t)w * h * 4);
        lv.dst_bytes = tx_compressed_size(r.format, w, h);
        lv.out_off = out;
        out += lv.dst_bytes;
        q->levels.push_back(lv);
        w = w > 1 ? w >> 1 : 1;
        h = h > 1 ? h >> 1 : 1;
    }
    for (Level &lv : q->levels) {
        lv.dst_off = off;
        off += align_up(lv.dst_bytes);
    }
    q->footprint = off;
    q->next_block.assign(q->levels.size(), 0);
    for (const Level &lv : q->levels) q->unassigned += lv.nblocks;
}

void finish_cancelled(tx_server *s, Request *q) {  // caller holds s->mu
    q->status = TX_ERR_CANCELLED;
    q->t_done = now_us();
    q->finished.store(true);
    s->cv_done.notify_all();
}

// Device memory an admission may take now: the device's free memory plus
// what the pool holds that no request uses, less the headroom.
cudaError_t hbm_available(tx_server *s, size_t *avail) {
    size_t fr = 0, total = 0;
    cudaError_t e = cudaMemGetInfo(&fr, &total);
    if (e != cudaSuccess) return e;
    uint64_t reserved = 0, used = 0;  // the attributes are 64-bit values
    if ((e = cudaMemPoolGetAttribute(s->pool, cudaMemPoolAttrReservedMemCurrent, &reserved)) != cudaSuccess) return e;
    if ((e = cudaMemPoolGetAttribute(s->pool, cudaMemPoolAttrUsedMemCurrent, &used)) != cudaSuccess) return e;
    const size_t a = fr + (size_t)(reserved > used ? reserved - used : 0);
    *avail = a > kHbmHeadroom ? a - kHbmHeadroom : 0;
    return cudaSuccess;
}

// Admit the head of the waiting line while the budget and the device's free
// memory allow (FIFO: a request that does not fit holds back the ones behind
// it, so a large request is never starved by small ones).
int admit(tx_server *s) {
    bool queried = false;
    size_t avail = 0;
    while (!s->waiting.empty()) {
        Request *q = s->waiting.front();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (q->cancel) {
                s->waiting.pop_front();
                finish_cancelled(s, q);
                continue;
            }
        }
        if (s->held + q->footprint > s->cfg.memory_budget) break;
        cudaError_t e;
        if (!queried || avail < q->footprint) {
            // while the head waits for memory that another process holds, ask
            // the driver at most every 200 us (a completion of ours resets it)
            if (q->hbm_deferred && now_us() < s->hbm_retry_at) break;
            if ((e = hbm_available(s, &avail)) != cudaSuccess) return fail_server(e);
            queried = true;
        }
        if (avail < q->footprint) {
            s->hbm_retry_at = now_us() + 200.0;
            if (!q->hbm_deferred) {
                q->hbm_deferred = true;
                std::lock_guard<std::mutex> lk(s->mu);
                s->hbm_waits++;
            }
            break;
        }
        void *ptr = nullptr;
        e = cudaMallocFromPoolAsync(&ptr, q->footprint, s->pool, s->s_load);
        if (e == cudaErrorMemoryAllocation) {  // lost a race for the memory: retry later
            cudaGetLastError();
            avail = 0;
            break;
        }
        if (e != cudaSuccess) return fail_server(e);
        avail -= q->footprint;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (q->cancel) {  // cancelled between the check and the allocation
                if ((e = cudaFreeAsync(ptr, s->s_load)) != cudaSuccess) return fail_server(e);
                s->waiting.pop_front();
                finish_cancelled(s, q);
                continue;
            }
            q->admitted = true;
            s->held += q->footprint;
            s->held_high = std::max(s->held_high, s->held);
        }
        nvtxRangePushA("tx_server admit");
        s->waiting.pop_front();
        q->dev = static_cast<uint8_t *>(ptr);
        q->t_admit = now_us();
        q->state = Request::LOADING;
        uint8_t *base = q->dev;
        const Level &l0 = q->levels[0];
        e = cudaMemcpyAsync(base + l0.src_off, q->r.rgba, (size_t)l0.w * l0.h * 4, cudaMemcpyHostToDevice, s->s_load);
        if (e != cudaSuccess) return fail_server(e);
        for (size_t l = 1; l < q->levels.size(); ++l) {
            const Level &a = q->levels[l - 1], &b = q->levels[l];
            tx_mip_job job{base + a.src_off, (size_t)a.w * 4, a.w, a.h, 4, base + b.src_off, (size_t)b.w * 4};
            int rc = tx_mip_batch_device(&job, 1, s->s_load);
            if (rc != TX_OK) return rc;
        }
        if ((e = cudaEventRecord(q->ready_ev, s->s_load)) != cudaSuccess) return fail_server(e);
        s->live.push_back(q);
        nvtxRangePop();
    }
    return TX_OK;
}

// Assemble one step from the ready requests and enqueue it.
int schedule_step(tx_server *s) {
    Step &st = s->steps[s->next_step];
    if (st.busy) return TX_OK;
    std::vector<Request *> ready;
    for (Request *q : s->live)
        if (q->state == Request::ACTIVE && q->unassigned > 0) ready.push_back(q);
    if (ready.empty()) return TX_OK;
    const uint32_t cap = s->cfg.step_blocks;
    const size_t share = std::max<size_t>(s->cfg.min_share, cap / ready.size());
    uint32_t n_items = 0, n_lane = 0;
    std::vector<uint2> lane_units, class_units[tx::kTeamClasses];
    const uint32_t lane_span = 32u * (uint32_t)s->cfg.tuning.lane_blocks_per_lane;
    const uint32_t team_span = (uint32_t)s->cfg.tuning.team_blocks_per_unit;
    size_t budget = cap;
    st.finishing.clear();
    const size_t start = s->rr % ready.size();
    for (size_t k = 0; k < ready.size() && budget > 0 && n_items < s->max_items; ++k) {
        Request *q = ready[(start + k) % ready.size()];
        size_t take = std::min(share, budget);
        for (size_t l = 0; l < q->levels.size() && take > 0 && n_items < s->max_items; ++l) {
            Level &lv = q->levels[l];
            uint32_t &nb = q->next_block[l];
            if (nb >= lv.nblocks) continue;
            const uint32_t n = (uint32_t)std::min<size_t>(take, lv.nblocks - nb);
            tx_batch_item it{};
            it.src = q->dev + lv.src_off;
            it.src_pitch = (size_t)lv.w * 4;
            it.width = lv.w;
            it.height = lv.h;
            it.format = q->r.format;
            it.channels = 4;
            it.params = q->r.params;
            it.dst = q->dev + lv.dst_off;
            tx::fill_batch_item(it, &st.h_items[n_items]);
            const tx::BatchItem &d = st.h_items[n_items];
            const bool lane = d.kind == tx::KIND_ALPHA || d.kind == tx::KIND_RANGE;
            const uint32_t span = lane ? lane_span : team_span;
            auto &dst = lane ? lane_units : class_units[tx::team_class(d.format, d.kind)];
            for (uint32_t f = nb; f < nb + n; f += span) dst.push_back(make_uint2(n_items, f));
            // a unit may run past this step's share; the kernels stop at the level's end,
            // so round the share up to whole units
            const uint32_t done = std::min<uint32_t>(lv.nblocks - nb, ((n + span - 1) / span) * span);
            nb += done;
            q->unassigned -= done;
            take -= std::min<size_t>(take, done);
            budget -= std::min<size_t>(budget, done);
            ++n_items;
        }
        q->steps++;
        if (q->unassigned == 0) st.finishing.push_back(q);
    }
    s->rr = start + 1;
    n_lane = (uint32_t)lane_units.size();
    uint32_t team_counts[tx::kTeamClasses];
    uint32_t total = n_lane;
    for (int c = 0; c < tx::kTeamClasses; ++c) {
        team_counts[c] = (uint32_t)class_units[c].size();
        total += team_counts[c];
    }
    if (total > s->max_units) return TX_ERR_INVALID_ARGUMENT;  // cannot happen: units <= step_blocks + items
    std::memcpy(st.h_units, lane_units.data(), n_lane * sizeof(uint2));
    for (uint32_t c = 0, off = n_lane; c < (uint32_t)tx::kTeamClasses; off += team_counts[c], ++c)
        std::memcpy(st.h_units + off, class_units[c].data(), team_counts[c] * sizeof(uint2));
    cudaError_t e;
    nvtxRangePushA("tx_server step");
    if ((e = cudaEventRecord(st.start, s->s_comp)) != cudaSuccess) return fail_server(e);
    if ((e = cudaMemcpyAsync(st.d_items, st.h_items, n_items * sizeof(tx::BatchItem), cudaMemcpyHostToDevice,
                             s->s_comp)) != cudaSuccess)
        return fail_server(e);
    if ((e = cudaMemcpyAsync(st.d_units, st.h_units, total * sizeof(uint2), cudaMemcpyHostToDevice, s->s_comp)) !=
        cudaSuccess)
        return fail_server(e);
    if ((e = cudaMemsetAsync(st.d_counters, 0, tx::kBatchCounters * sizeof(uint32_t), s->s_comp)) != cudaSuccess) return fail_server(e);
    if ((e = tx::launch_batch_queues(st.d_items, st.d_units, n_lane, lane_span / 32, st.d_units + n_lane,
                                     team_counts, team_span, st.d_counters, s->sm_count, s->cfg.tuning,
                                     s->s_comp)) != cudaSuccess)
        return fail_server(e);
    if ((e = cudaEventRecord(st.done, s->s_comp)) != cudaSuccess) return fail_server(e);
    nvtxRangePop();
    st.busy = true;
    s->next_step ^= 1;
    s->step_count++;
    return TX_OK;
}

// Retire finished steps: start the device->host copies of requests that are complete.
int retire_steps(tx_server *s) {
    for (int i = 0; i < 2; ++i) {
        Step &st = s->steps[(s->next_step + i) & 1];  // oldest first
        if (!st.busy) continue;
        cudaError_t e = cudaEventQuery(st.done);
        if (e == cudaErrorNotReady) return TX_OK;  // steps complete in order
        if (e != cudaSuccess) return fail_server(e);
        float ms = 0.0f;
        if ((e = cudaEventElapsedTime(&ms, st.start, st.done)) != cudaSuccess) return fail_server(e);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->busy_us += (double)ms * 1e3;
        }
        for (Request *q : st.finishing) {
            uint8_t *base = q->dev;
            if ((e = cudaStreamWaitEvent(s->s_store, st.done, 0)) != cudaSuccess) return fail_server(e);
            for (const Level &lv : q->levels) {
                if (lv.dst_bytes == 0) continue;
                if ((e = cudaMemcpyAsync(q->r.output + lv.out_off, base + lv.dst_off, lv.dst_bytes, cudaMemcpyDeviceToHost,
                                         s->s_store)) != cudaSuccess)
                    return fail_server(e);
            }
            if ((e = cudaEventRecord(q->done_ev, s->s_store)) != cudaSuccess) return fail_server(e);
            q->state = Request::DRAINING;
        }
        st.finishing.clear();
        st.busy = false;
    }
    return TX_OK;
}

// Promote loaded requests and complete drained ones.
int progress(tx_server *s, bool *completed_any) {
    *completed_any = false;
    for (size_t i = 0; i < s->live.size();) {
        Request *q = s->live[i];
        if (q->state == Request::LOADING) {
            cudaError_t e = cudaEventQuery(q->ready_ev);
            if (e == cudaSuccess) {
                q->state = Request::ACTIVE;
                if (q->unassigned == 0) {  // an empty image: nothing to compress
                    q->state = Request::DRAINING;
                    if ((e = cudaEventRecord(q->done_ev, s->s_load)) != cudaSuccess) return fail_server(e);
                }
            } else if (e != cudaErrorNotReady) {
                return fail_server(e);
            }
        } else if (q->state == Request::DRAINING) {
            cudaError_t e = cudaEventQuery(q->done_ev);
            if (e == cudaSuccess) {
                // back to the pool behind the copies (done_ev has completed)
                if ((e = cudaFreeAsync(q->dev, s->s_store)) != cudaSuccess) return fail_server(e);
                q->dev = nullptr;
                s->hbm_retry_at = 0;  // memory came back: a waiting head may fit now
                std::lock_guard<std::mutex> lk(s->mu);
                s->held -= q->footprint;
                q->t_done = now_us();
                q->state = Request::DONE;
                q->finished.store(true);
                s->n_completed++;
                s->live.erase(s->live.begin() + (long)i);
                *completed_any = true;
                continue;
            } else if (e != cudaErrorNotReady) {
                return fail_server(e);
            }
        }
        ++i;
    }
    return TX_OK;
}

void fail_all(tx_server *s, int rc) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->fatal = rc;
    for (auto &kv : s->requests) {
        Request *q = kv.second;
        if (!q->finished.load()) {
            q->status = rc;
            q->t_done = now_us();
            q->finished.store(true);
        }
    }
    s->submitted.clear();
    s->cv_done.notify_all();
}

void worker_main(tx_server *s) {
    cudaSetDevice(s->device);
    bool idle = false;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->fatal != TX_OK) return;
            if (s->submitted.empty() && s->waiting.empty() && s->live.empty()) {
                if (s->stopping) return;
                if (!idle) {  // nothing admitted: give the pool's memory back to the device
                    cudaMemPoolTrimTo(s->pool, 0);
                    idle = true;
                }
                s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
            } else {
                idle = false;
            }
            while (!s->submitted.empty()) {
                s->waiting.push_back(s->submitted.front());
                s->submitted.pop_front();
            }
        }
        int rc = admit(s);
        bool done = false;
        if (rc == TX_OK) rc = progress(s, &done);
        if (rc == TX_OK) rc = retire_steps(s);
        if (rc == TX_OK) rc = schedule_step(s);
        if (rc == TX_OK) rc = schedule_step(s);  // keep two steps in flight
        if (rc != TX_OK) {
            fail_all(s, rc);
            return;
        }
        if (done) s->cv_done.notify_all();
        // nothing to launch: let the GPU work before polling again
        if (s->steps[0].busy && s->steps[1].busy) std::this_thread::sleep_for(std::chrono::microseconds(20));
        else if (!s->live.empty()) std::this_thread::sleep_for(std::chrono::microseconds(5));
    }
}

void destroy_resources(tx_server *s) {
    for (Step &st : s->steps) {
        cudaFree(st.d_items);
        cudaFree(st.d_units);
        cudaFree(st.d_counters);
        cudaFreeHost(st.h_items);
        cudaFreeHost(st.h_units);
        if (st.start) cudaEventDestroy(st.start);
        if (st.done) cudaEventDestroy(st.done);
    }
    if (s->pool) cudaMemPoolDestroy(s->pool);
    if (s->s_load) cudaStreamDestroy(s->s_load);
    if (s->s_comp) cudaStreamDestroy(s->s_comp);
    if (s->s_store) cudaStreamDestroy(s->s_store);
}

}  // namespace

extern "C" {

size_t tx_chain_compressed_size(int format, uint32_t width, uint32_t height, int mips) {
    if (tx_block_size(format) == 0) return 0;
    const uint32_t n = mips ? tx_mip_count(width, height) : (width && height ? 1u : 0u);
    size_t total = 0;
    for (uint32_t l = 0; l < n; ++l) {
        total += tx_compressed_size(format, width, height);
        width = width > 1 ? width >> 1 : 1;
        height = height > 1 ? height >> 1 : 1;
    }
    return total;
}

void tx_server_default_config(tx_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->memory_budget = (size_t)40 << 30;
    c->step_blocks = 1u << 20;
    c->min_share = 1u << 14;
    tx_batch_default_tuning(&c->tuning);
}

int tx_server_create(const tx_server_config *config, tx_server **out) {
    if (!out) return TX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    tx_server_config cfg;
    tx_server_default_config(&cfg);
    if (config) {
        if (config->memory_budget) cfg.memory_budget = config->memory_budget;
        if (config->step_blocks) cfg.step_blocks = config->step_blocks;
        if (config->min_share) cfg.min_share = config->min_share;
        tx_batch_tuning t = cfg.tuning;
        const tx_batch_tuning &u = config->tuning;
        if (u.team_lanes == 16 || u.team_lanes == 32) t.team_lanes = u.team_lanes;
        if (u.team_threads_per_cta >= 64 && u.team_threads_per_cta <= 256 && u.team_threads_per_cta % 32 == 0)
            t.team_threads_per_cta = u.team_threads_per_cta;
        if (u.team_ctas_per_sm >= 1 && u.team_ctas_per_sm <= 16) t.team_ctas_per_sm = u.team_ctas_per_sm;
        if (u.team_blocks_per_unit >= 1 && u.team_blocks_per_unit <= 64) t.team_blocks_per_unit = u.team_blocks_per_unit;
        if (u.team_blocks_in_flight >= 1 && u.team_blocks_in_flight <= 3) t.team_blocks_in_flight = u.team_blocks_in_flight;
        if (u.lane_ctas_per_sm >= 1 && u.lane_ctas_per_sm <= 16) t.lane_ctas_per_sm = u.lane_ctas_per_sm;
        if (u.lane_blocks_per_lane >= 1 && u.lane_blocks_per_lane <= 64) t.lane_blocks_per_lane = u.lane_blocks_per_lane;
        cfg.tuning = t;
    }
    if (cfg.step_blocks < 1024 || cfg.step_blocks > (1u << 26)) return TX_ERR_INVALID_ARGUMENT;
    int rc = tx_internal_ensure_device();
    if (rc != TX_OK) return rc;
    tx_server *s = new (std::nothrow) tx_server();
    if (!s) return TX_ERR_OUT_OF_MEMORY;
    s->cfg = cfg;
    cudaGetDevice(&s->device);
    cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
    s->max_items = 65536;
    s->max_units = cfg.step_blocks + s->max_items * 2;
    // requests' device memory: a pool of the server's own, which keeps up to
    // the budget mapped between requests and is trimmed when the server idles
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    cudaError_t e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = cfg.memory_budget;
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_load, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_store, cudaStreamNonBlocking);
    for (Step &st : s->steps) {
        if (e == cudaSuccess) e = cudaMalloc(&st.d_items, s->max_items * sizeof(tx::BatchItem));
        if (e == cudaSuccess) e = cudaMalloc(&st.d_units, s->max_units * sizeof(uint2));
        if (e == cudaSuccess) e = cudaMalloc(&st.d_counters, tx::kBatchCounters * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMallocHost(&st.h_items, s->max_items * sizeof(tx::BatchItem));
        if (e == cudaSuccess) e = cudaMallocHost(&st.h_units, s->max_units * sizeof(uint2));
        if (e == cudaSuccess) e = cudaEventCreate(&st.start);
        if (e == cudaSuccess) e = cudaEventCreate(&st.done);
    }
    if (e != cudaSuccess) {
        destroy_resources(s);
        delete s;
        return fail_server(e);
    }
    s->worker = std::thread(worker_main, s);
    *out = s;
    return TX_OK;
}

int tx_server_submit(tx_server *s, const tx_server_request *req, uint64_t *id) {
    if (!s || !req || !id) return TX_ERR_INVALID_ARGUMENT;
    if (tx_block_size(req->format) == 0) return TX_ERR_INVALID_FORMAT;
    if (req->params.algorithm < TX_RANGE_FIT || req->params.algorithm > TX_ITERATIVE_CLUSTER_FIT)
        return TX_ERR_INVALID_ARGUMENT;
    if (req->width == 0 || req->height == 0 || !req->rgba) return TX_ERR_INVALID_ARGUMENT;
    if (tx_num_blocks(req->width) * tx_num_blocks(req->height) > tx::kMaxBatchLevelBlocks)
        return TX_ERR_INVALID_ARGUMENT;
    if (req->output_len < tx_chain_compressed_size(req->format, req->width, req->height, req->mips))
        return TX_ERR_OUTPUT_TOO_SMALL;
    if (!req->output) return TX_ERR_INVALID_ARGUMENT;
    Request *q = new (std::nothrow) Request();
    if (!q) return TX_ERR_OUT_OF_MEMORY;
    q->r = *req;
    plan_levels(q);
    if (q->footprint > s->cfg.memory_budget) {
        delete q;
        return TX_ERR_OUT_OF_MEMORY;  // could never be admitted
    }
    if (cudaEventCreateWithFlags(&q->ready_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&q->done_ev, cudaEventDisableTiming) != cudaSuccess) {
        if (q->ready_ev) cudaEventDestroy(q->ready_ev);
        delete q;
        return TX_ERR_CUDA;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->fatal != TX_OK) {
            cudaEventDestroy(q->ready_ev);
            cudaEventDestroy(q->done_ev);
            delete q;
            return s->fatal;
        }
        if (s->stopping) {
            cudaEventDestroy(q->ready_ev);
            cudaEventDestroy(q->done_ev);
            delete q;
            return TX_ERR_CANCELLED;
        }
        q->id = s->next_id++;
        q->t_submit = now_us();
        s->requests[q->id] = q;
        s->submitted.push_back(q);
        s->n_submitted++;
        *id = q->id;
    }
    s->cv_work.notify_one();
    return TX_OK;
}

int tx_server_wait(tx_server *s, uint64_t id, int timeout_ms, tx_server_result *res) {
    if (!s) return TX_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return TX_ERR_INVALID_ARGUMENT;
    Request *q = it->second;
    auto pred = [&] { return q->finished.load(); };
    if (timeout_ms < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return TX_ERR_TIMEOUT;
    if (res) {
        res->status = q->status;
        res->latency_us = q->t_done - q->t_submit;
        res->queue_us = q->t_admit > 0 ? q->t_admit - q->t_submit : q->t_done - q->t_submit;
        res->blocks = 0;
        for (const Level &lv : q->levels) res->blocks += lv.nblocks;
        res->levels = (uint32_t)q->levels.size();
        res->steps = q->steps;
    }
    const int status = q->status;
    s->requests.erase(it);
    lk.unlock();
    cudaEventDestroy(q->ready_ev);
    cudaEventDestroy(q->done_ev);
    delete q;
    return status;
}

int tx_server_cancel(tx_server *s, uint64_t id) {
    if (!s) return TX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->requests.find(id);
    if (it == s->requests.end()) return TX_ERR_INVALID_ARGUMENT;
    Request *q = it->second;
    if (q->finished.load()) return q->status == TX_ERR_CANCELLED ? TX_OK : TX_ERR_BUSY;
    if (q->admitted) return TX_ERR_BUSY;  // already in device memory: it runs to completion
    for (auto sub = s->submitted.begin(); sub != s->submitted.end(); ++sub) {
        if (*sub == q) {  // the worker has not seen it yet
            s->submitted.erase(sub);
            finish_cancelled(s, q);
            return TX_OK;
        }
    }
    q->cancel = true;  // waiting for memory: the worker drops it at admission
    return TX_OK;
}

int tx_server_get_stats(tx_server *s, tx_server_stats *out) {
    if (!s || !out) return TX_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    out->submitted = s->n_submitted;
    out->completed = s->n_completed;
    out->steps = s->step_count;
    out->memory_budget = s->cfg.memory_budget;
    out->held_high_water = s->held_high;
    out->busy_us = s->busy_us;
    out->hbm_deferrals = s->hbm_waits;
    return TX_OK;
}

void tx_server_destroy(tx_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaStreamSynchronize(s->s_load);
    cudaStreamSynchronize(s->s_comp);
    cudaStreamSynchronize(s->s_store);
    for (Request *q : s->live)  // only after a fatal error: requests that still hold memory
        if (q->dev) cudaFreeAsync(q->dev, s->s_store);
    cudaStreamSynchronize(s->s_store);
    for (auto &kv : s->requests) {
        cudaEventDestroy(kv.second->ready_ev);
        cudaEventDestroy(kv.second->done_ev);
        delete kv.second;
    }
    destroy_resources(s);
    delete s;
}

}  // extern "C"
