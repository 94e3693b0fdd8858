// server.cpp -- continuous-batching request loop over resident stream pools.
//
// The streams of a 32-bit and a 64-bit pool stay resident on the device.
// Clients submit requests (stream, skip, count, output kind, destination);
// a scheduler thread admits them into batches and runs each batch as one
// persistent launch (the batched kernels, through the public plan API):
//   - up to `slots` batches are in flight at once, each on its own CUDA
//     stream, so a batch admitted while others run overlaps them on the GPU;
//   - a request is admitted when a slot is free and its output fits in the
//     device output arena (the memory budget); admission is first-come,
//     first-served; a request whose stream has work on the GPU waits, and
//     requests of one stream run in submission order (several may share a
//     batch), each seeing the stream where the previous one left it;
//   - a request's skip is done by generation when short and by a GF(2) jump
//     when long (mtgp_work_item_t);
//   - when a batch completes, results are copied to the callers'
//     destinations (device or host memory) and their arena space is
//     returned; a request without a destination keeps its result in the
//     arena (zero copy, read through mtgp_server_result) until it is
//     released; the latency (completion - submission) is recorded.
// A request's output depends only on its stream's position, so it is the
// same alone and in any mix.
//
// Threads: the scheduler thread only admits (first-come-first-served, the
// arena, the stream states) and hands each batch to a free slot; every slot
// has a worker thread that plans and launches its batch (the pools' plans
// can be made on several threads at once), waits for it on the GPU and
// retires it (latencies, arena space, stream states).  So the host work of
// up to `slots` batches runs in parallel instead of on one thread.  A batch
// is admitted (everything admissible, up to max_batch) when a slot is free
// and no other batch is being planned (low load: a lone request goes
// straight to the GPU; under load the next batch collects what arrives
// while one is planned), or when a quarter of a full batch is waiting:
// only then are several batches planned at once.  Admitting at every chance instead splits
// the work into many small launches and keeps the scheduler scanning a
// backlog that is mostly requests of streams already on the GPU.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "server_core.h"

namespace {

using Clock = std::chrono::steady_clock;

// Skips at least this long are done by a GF(2) jump in the batched kernel
// (the planner's threshold for MEXP 11213 and 23209).
constexpr uint64_t kJumpSkip = uint64_t(1) << 17;

using Req = mtgp::ServeReq;
using mtgp::Arena;

struct Slot {
    cudaStream_t cs = nullptr;
    cudaEvent_t ev = nullptr;
    mtgp_gpu_plan_t *plan[2] = {nullptr, nullptr};
    std::vector<Req> reqs;  // the batch (owned by the worker while busy)
    bool busy = false;      // holds a batch: handed over, launching or on the GPU
    bool assigned = false;  // handed over, not yet taken by the worker
    bool planning = false;  // handed over and not yet launched
    std::thread th;         // the slot's worker
    std::condition_variable cv;
};

}  // namespace

struct mtgp_server {
    mtgp32_gpu_pool_t *p32 = nullptr;
    mtgp64_gpu_pool_t *p64 = nullptr;
    int nstreams[2] = {0, 0};
    int device = 0;
    unsigned char *d_arena = nullptr;
    Arena arena;
    std::vector<std::unique_ptr<Slot>> slots;
    int max_batch = 4096;
    int nplanning = 0;  // slots whose batch is handed over and not yet launched
    // set when admission may take more: a submission, a retired batch or
    // released space since the scheduler's last admission pass
    bool dirty = false;
    bool sched_waiting = false;  // the scheduler sleeps on cv (a submission wakes it)
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<Req> pending;
    std::vector<char> busy[2];
    std::thread th;
    std::atomic<bool> stop{false};
    uint64_t submitted = 0, completed = 0, bytes_done = 0, batches = 0;
    // seconds and MTGP_* status by ticket - 1 (latency -1 = not done); deques,
    // so that millions of tickets never make a submit (under the lock the
    // scheduler needs) copy the whole history to grow
    std::deque<double> latency;
    std::deque<int> status;
    std::map<uint64_t, std::pair<uint64_t, uint64_t>> kept;  // ticket -> (offset, bytes)
    // scheduler time (s): admission, planning + launch, retiring, idle waits
    // [4]: the planning part of [1] (pool_plan / pool_replan)
    double prof[5] = {0, 0, 0, 0, 0};
    Clock::time_point t0;

    int enqueue(int pool, uint32_t stream, int kind, uint64_t skip, uint64_t count, void *dst,
                bool keep, uint64_t *ticket);
    int enqueueLocked(int pool, uint32_t stream, int kind, uint64_t skip, uint64_t count,
                      void *dst, bool keep, uint64_t *ticket);

    void loop();
    void work(Slot &sl);
    int launch(Slot &sl, std::vector<Req> &reqs, double *plan_s);
    int launchBatch(Slot &sl, std::vector<Req> &reqs, double *plan_s);
};

int mtgp_server::launch(Slot &sl, std::vector<Req> &reqs, double *plan_s) {
    const int rc = launchBatch(sl, reqs, plan_s);
    // work already queued for this batch must end before its arena space is
    // handed to another batch
    if (rc) cudaStreamSynchronize(sl.cs);
    return rc;
}

int mtgp_server::launchBatch(Slot &sl, std::vector<Req> &reqs, double *plan_s) {
    std::vector<mtgp_work_item_t> items[2];
    for (const Req &r : reqs) {
        mtgp_work_item_t it{};
        it.stream = r.stream;
        it.kind = r.kind;
        it.count = r.count;
        it.out_offset = r.off;
        it.skip = r.skip;
        items[r.pool].push_back(it);
    }
    for (int p = 0; p < 2; p++) {
        if (items[p].empty()) continue;
        int rc;
        const int n = (int)items[p].size();
        const Clock::time_point tp = Clock::now();
        if (!sl.plan[p]) {
            rc = p == 0 ? mtgp32_gpu_pool_plan(p32, items[p].data(), n, &sl.plan[p])
                        : mtgp64_gpu_pool_plan(p64, items[p].data(), n, &sl.plan[p]);
        } else {
            rc = p == 0 ? mtgp32_gpu_pool_replan(p32, items[p].data(), n, sl.plan[p])
                        : mtgp64_gpu_pool_replan(p64, items[p].data(), n, sl.plan[p]);
        }
        *plan_s += std::chrono::duration<double>(Clock::now() - tp).count();
        if (!rc) rc = mtgp_gpu_plan_launch(sl.plan[p], d_arena, sl.cs);
        if (rc) return rc;
    }
    for (const Req &r : reqs) {
        if (!r.dst || !r.bytes) continue;
        cudaError_t e = cudaMemcpyAsync(r.dst, d_arena + r.off, r.bytes, cudaMemcpyDefault, sl.cs);
        if (e != cudaSuccess) return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaError_t e = cudaEventRecord(sl.ev, sl.cs);
    if (e != cudaSuccess) return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    return MTGP_OK;
}

void mtgp_server::loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    std::vector<Req> take;
    while (!stop.load()) {
        bool progressed = false;
        Slot *fs = nullptr;
        for (auto &sp : slots)
            if (!sp->busy) {
                fs = sp.get();
                break;
            }
        if (fs && dirty && !pending.empty() &&
            (nplanning == 0 || pending.size() >= (size_t)std::max(1, max_batch / 4))) {
            dirty = false;
            const Clock::time_point ta = Clock::now();
            mtgp::admitBatch(pending, busy, arena, max_batch, kJumpSkip, &take,
                             4 * (size_t)max_batch);
            prof[0] += std::chrono::duration<double>(Clock::now() - ta).count();
            if (!take.empty()) {
                fs->reqs.swap(take);
                fs->busy = fs->assigned = fs->planning = true;
                nplanning++;
                batches++;
                fs->cv.notify_one();
                dirty = true;  // another free slot may take more
                progressed = true;
            }
        }
        if (!progressed) {
            // woken by a submission, a retired batch or released space
            const Clock::time_point ti = Clock::now();
            sched_waiting = true;
            cv.wait_for(lk, std::chrono::milliseconds(1));
            sched_waiting = false;
            prof[3] += std::chrono::duration<double>(Clock::now() - ti).count();
        }
    }
}

void mtgp_server::work(Slot &sl) {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        sl.cv.wait(lk, [&] { return sl.assigned || stop.load(); });
        if (!sl.assigned) break;  // stopping
        sl.assigned = false;
        lk.unlock();
        // plan and launch, then wait for the batch: a short spin, so that
        // the retire follows a short batch closely, then a blocking wait
        // (the event is a blocking-sync one), so that long batches hold no
        // core
        const Clock::time_point tl = Clock::now();
        double plan_s = 0;
        const int rc = launch(sl, sl.reqs, &plan_s);
        const Clock::time_point tw = Clock::now();
        lk.lock();
        sl.planning = false;
        nplanning--;
        dirty = true;  // the next batch may be admitted now
        cv.notify_one();
        lk.unlock();
        cudaError_t q = cudaSuccess;
        if (!rc) {
            q = cudaEventQuery(sl.ev);
            while (q == cudaErrorNotReady &&
                   Clock::now() - tw < std::chrono::microseconds(100)) {
                std::this_thread::yield();
                q = cudaEventQuery(sl.ev);
            }
            if (q == cudaErrorNotReady) q = cudaEventSynchronize(sl.ev);
        }
        const Clock::time_point now = Clock::now();
        lk.lock();
        prof[1] += std::chrono::duration<double>(tw - tl).count();
        prof[4] += plan_s;
        const int st = rc ? rc : q == cudaSuccess ? MTGP_OK : MTGP_ERR_CUDA;
        for (const Req &r : sl.reqs) {
            latency[r.ticket - 1] = rc ? 0 : std::chrono::duration<double>(now - r.t_submit).count();
            status[r.ticket - 1] = st;
            if (!st && r.keep && r.bytes)
                kept[r.ticket] = {r.off, r.bytes};
            else
                arena.release(r.off, r.bytes);
            busy[r.pool][r.stream] = mtgp::kStreamFree;
            completed++;
            if (!st) bytes_done += r.bytes;
        }
        sl.reqs.clear();
        sl.busy = false;
        dirty = true;
        prof[2] += std::chrono::duration<double>(Clock::now() - now).count();
        cv.notify_one();
        cv_done.notify_all();
    }
}

extern "C" {

int mtgp_server_create(mtgp_server_t **out, mtgp32_gpu_pool_t *p32, mtgp64_gpu_pool_t *p64,
                       uint64_t budget_bytes, int slots, int max_batch) {
    if (!out || (!p32 && !p64) || budget_bytes < 256 || slots < 1 || max_batch < 1)
        return mtgp::recordError(MTGP_ERR_INVALID, "bad server arguments");
    *out = nullptr;
    mtgp_server *s = new (std::nothrow) mtgp_server();
    if (!s) return mtgp::recordError(MTGP_ERR_ALLOC, "server allocation");
    s->p32 = p32;
    s->p64 = p64;
    s->nstreams[0] = p32 ? mtgp32_gpu_pool_size(p32) : 0;
    s->nstreams[1] = p64 ? mtgp64_gpu_pool_size(p64) : 0;
    s->busy[0].assign(s->nstreams[0], 0);
    s->busy[1].assign(s->nstreams[1], 0);
    s->max_batch = max_batch;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = mtgp::devMalloc(&s->d_arena, budget_bytes);
    if (e != cudaSuccess) {
        delete s;
        return mtgp::recordError(MTGP_ERR_ALLOC, cudaGetErrorString(e));
    }
    s->arena.init(budget_bytes);
    for (int k = 0; k < slots; k++) {
        s->slots.emplace_back(new (std::nothrow) Slot());
        Slot *sl = s->slots.back().get();
        if (!sl) {
            s->slots.pop_back();
            e = cudaErrorMemoryAllocation;
            break;
        }
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl->cs, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming | cudaEventBlockingSync);
    }
    if (e != cudaSuccess) {
        mtgp_server_destroy(s);
        return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    }
    s->t0 = Clock::now();
    for (auto &sp : s->slots) {
        Slot *sl = sp.get();
        sl->th = std::thread([s, sl] { s->work(*sl); });
    }
    s->th = std::thread([s] { s->loop(); });
    *out = s;
    return MTGP_OK;
}

int mtgp_server::enqueue(int pool, uint32_t stream, int kind, uint64_t skip, uint64_t count,
                         void *dst, bool keep, uint64_t *ticket) {
    std::lock_guard<std::mutex> lk(mu);
    return enqueueLocked(pool, stream, kind, skip, count, dst, keep, ticket);
}

// enqueue with mu held (replay submits all requests that are due under one
// lock); the scheduler is woken only when it sleeps, so a burst of
// submissions costs no wake-up each.
int mtgp_server::enqueueLocked(int pool, uint32_t stream, int kind, uint64_t skip,
                               uint64_t count, void *dst, bool keep, uint64_t *ticket) {
    if (!ticket) return mtgp::recordError(MTGP_ERR_INVALID, "null ticket");
    if (pool < 0 || pool > 1 || stream >= (uint32_t)nstreams[pool])
        return mtgp::recordError(MTGP_ERR_INVALID, "no such pool or stream");
    if (kind < -1 || kind > 4) return mtgp::recordError(MTGP_ERR_INVALID, "unknown output kind");
    const uint64_t esz = pool == 0 ? 4u : 8u;
    if (kind >= 0 && count > ~uint64_t(0) / esz)
        return mtgp::recordError(MTGP_ERR_BUDGET, "request larger than the device budget");
    const uint64_t bytes = kind < 0 ? 0 : count * esz;
    if (Arena::round(bytes) > arena.size())
        return mtgp::recordError(MTGP_ERR_BUDGET, "request larger than the device budget");
    Req r{};
    r.ticket = ++submitted;
    r.pool = pool;
    r.stream = stream;
    r.kind = kind;
    r.skip = skip;
    r.count = count;
    r.bytes = bytes;
    r.dst = dst;
    r.keep = keep && !dst;
    r.t_submit = Clock::now();
    latency.push_back(-1.0);
    status.push_back(1);
    pending.push_back(r);
    *ticket = r.ticket;
    dirty = true;
    if (sched_waiting) cv.notify_one();
    return MTGP_OK;
}

int mtgp_server_submit(mtgp_server_t *s, int pool, uint32_t stream, int kind, uint64_t skip,
                       uint64_t count, void *dst, uint64_t *ticket) {
    if (!s) return mtgp::recordError(MTGP_ERR_INVALID, "null server");
    return s->enqueue(pool, stream, kind, skip, count, dst, true, ticket);
}

int mtgp_server_result(mtgp_server_t *s, uint64_t ticket, void **dev_ptr, uint64_t *bytes) {
    if (!s || !dev_ptr) return mtgp::recordError(MTGP_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->kept.find(ticket);
    if (it == s->kept.end())
        return mtgp::recordError(MTGP_ERR_INVALID, "no result held for this ticket");
    *dev_ptr = s->d_arena + it->second.first;
    if (bytes) *bytes = it->second.second;
    return MTGP_OK;
}

int mtgp_server_release(mtgp_server_t *s, uint64_t ticket) {
    if (!s) return mtgp::recordError(MTGP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->kept.find(ticket);
    if (it == s->kept.end())
        return mtgp::recordError(MTGP_ERR_INVALID, "no result held for this ticket");
    s->arena.release(it->second.first, it->second.second);
    s->kept.erase(it);
    s->dirty = true;
    s->cv.notify_one();
    return MTGP_OK;
}

int mtgp_server_cancel(mtgp_server_t *s, uint64_t ticket) {
    if (!s) return mtgp::recordError(MTGP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto it = s->pending.begin(); it != s->pending.end(); ++it) {
        if (it->ticket != ticket) continue;
        s->latency[ticket - 1] = 0;
        s->status[ticket - 1] = MTGP_ERR_BUSY;  // cancelled before it ran
        s->completed++;
        s->pending.erase(it);
        s->cv_done.notify_all();
        return MTGP_OK;
    }
    return mtgp::recordError(MTGP_ERR_INVALID, "ticket is not pending");
}

int mtgp_server_wait(mtgp_server_t *s, uint64_t ticket, double timeout_s, int *status) {
    if (!s || ticket == 0) return mtgp::recordError(MTGP_ERR_INVALID, "bad wait");
    std::unique_lock<std::mutex> lk(s->mu);
    if (ticket > s->submitted) return mtgp::recordError(MTGP_ERR_INVALID, "unknown ticket");
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->latency[ticket - 1] >= 0; });
    if (!ok) return mtgp::recordError(MTGP_ERR_TIMEOUT, "request not done in time");
    if (status) *status = s->status[ticket - 1];
    return MTGP_OK;
}

int mtgp_server_drain(mtgp_server_t *s, double timeout_s) {
    if (!s) return mtgp::recordError(MTGP_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->completed == s->submitted; });
    return ok ? MTGP_OK : mtgp::recordError(MTGP_ERR_TIMEOUT, "requests still in flight");
}

int mtgp_server_results(mtgp_server_t *s, double *latency, int *status, uint64_t cap,
                        uint64_t *n) {
    if (!s) return mtgp::recordError(MTGP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t m = std::min<uint64_t>(cap, s->latency.size());
    for (uint64_t k = 0; k < m; k++) {
        if (latency) latency[k] = s->latency[k];
        if (status) status[k] = s->status[k];
    }
    if (n) *n = s->latency.size();
    return MTGP_OK;
}

int mtgp_server_stats(mtgp_server_t *s, uint64_t *completed, uint64_t *bytes, uint64_t *batches) {
    if (!s) return mtgp::recordError(MTGP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    if (completed) *completed = s->completed;
    if (bytes) *bytes = s->bytes_done;
    if (batches) *batches = s->batches;
    return MTGP_OK;
}

int mtgp_server_profile(mtgp_server_t *s, double *seconds, int n) {
    if (!s || (n > 0 && !seconds)) return mtgp::recordError(MTGP_ERR_INVALID, "bad profile");
    std::lock_guard<std::mutex> lk(s->mu);
    for (int k = 0; k < n && k < 5; k++) seconds[k] = s->prof[k];
    return MTGP_OK;
}

int mtgp_server_replay(mtgp_server_t *s, const mtgp_request_t *reqs, const double *arrival_s,
                       int n, double *wall_s) {
    if (!s || n < 0 || (n > 0 && (!reqs || !arrival_s)))
        return mtgp::recordError(MTGP_ERR_INVALID, "bad trace");
    const Clock::time_point start = Clock::now();
    auto due = [&](int k) {
        return start + std::chrono::duration_cast<Clock::duration>(
                           std::chrono::duration<double>(arrival_s[k]));
    };
    for (int k = 0; k < n;) {
        const Clock::time_point at = due(k);
        while (Clock::now() < at) {
            const auto left = at - Clock::now();
            if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left / 2);
        }
        // every request already due (at most 1024), under one lock
        std::lock_guard<std::mutex> lk(s->mu);
        const Clock::time_point now = Clock::now();
        const int k0 = k;
        do {
            uint64_t t = 0;
            const mtgp_request_t &r = reqs[k];
            int rc = s->enqueueLocked(r.pool, r.stream, r.kind, r.skip, r.count, r.dst, false, &t);
            if (rc) return rc;
            k++;
        } while (k < n && k - k0 < 1024 && due(k) <= now);
    }
    int rc = mtgp_server_drain(s, 600.0);
    if (wall_s) *wall_s = std::chrono::duration<double>(Clock::now() - start).count();
    return rc;
}

void mtgp_server_destroy(mtgp_server_t *s) {
    if (!s) return;
    if (s->th.joinable()) mtgp_server_drain(s, 600.0);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop.store(true);
        s->cv.notify_all();
        for (auto &sp : s->slots) sp->cv.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    for (auto &sp : s->slots)
        if (sp->th.joinable()) sp->th.join();
    for (auto &sp : s->slots) {
        Slot &sl = *sp;
        if (sl.cs) cudaStreamSynchronize(sl.cs);
        for (int p = 0; p < 2; p++) mtgp_gpu_plan_free(sl.plan[p]);
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.cs) cudaStreamDestroy(sl.cs);
    }
    cudaFree(s->d_arena);
    delete s;
}

}  // extern "C"
