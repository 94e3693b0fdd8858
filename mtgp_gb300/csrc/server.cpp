// server.cpp -- continuous-batching request loop over resident stream pools.
//
// The streams of a 32-bit and a 64-bit pool stay resident on the device.
// Clients submit requests (stream, skip, count, output kind, destination);
// a scheduler thread admits them into batches and runs each batch as one
// persistent launch per pool (the batched kernels, through the public plan
// API):
//   - up to `slots` batches are in flight at once, each on its own CUDA
//     streams (one per pool), so a batch admitted while others run overlaps
//     them on the GPU, and a batch's two pools run side by side;
//   - admission is first-come, first-served; requests of one stream run in
//     submission order, each seeing the stream where the previous one left
//     it.  Several may share a batch (run in order by the plan).  A stream
//     whose earlier requests are still on the GPU waits for them under a
//     light load (so that batches share no stream and run side by side);
//     under a backlog it joins the new batch, which the GPU then runs after
//     those batches: an event wait per earlier batch on the new batch's
//     CUDA stream of that pool, made once they are launched;
//   - a batch's outputs take one block of the device output arena (the
//     memory budget), placed in admission order (at admission if there is
//     room, else once the batch is planned);
//   - a request's skip is done by generation when short and by a GF(2) jump
//     when long (mtgp_work_item_t);
//   - when a batch completes, results are copied to the callers'
//     destinations (device or host memory) and its arena block is returned;
//     a request without a destination keeps its result in the arena (zero
//     copy, read through mtgp_server_result) until it is released; the
//     latency (completion - submission) is recorded.
// A request's output depends only on its stream's position, so it is the
// same alone and in any mix.
//
// Threads: the scheduler thread only admits (first-come-first-served, the
// streams' order) and hands each batch to a free slot; every slot has a
// worker thread that plans its batch (the pools' plans can be made on
// several threads at once), places it in the arena, launches it, waits for
// it on the GPU and retires it (latencies, arena space).  So the host work
// of up to `slots` batches runs in parallel, and the lock they share is held
// for a few word writes per request.  A batch is admitted (up to max_batch
// requests, under a backlog a quarter of what waits, and batchBytes of
// output) when a slot is free and no other batch is being planned (low load:
// a lone request goes straight to the GPU; under load the next batch
// collects what arrives while one is planned), or when a quarter of a full
// batch is waiting: only then are several batches planned at once.
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
    // a CUDA stream per pool: the two pools' parts of a batch run side by
    // side, each after the earlier batches' parts of the same pool
    cudaStream_t cs[2] = {nullptr, nullptr};
    cudaEvent_t ev = nullptr;    // the batch is complete (results copied)
    cudaEvent_t join = nullptr;  // the 64-bit pool's part is complete
    // the pool's kernels are done: its streams' windows are written
    cudaEvent_t dep_ev[2] = {nullptr, nullptr};
    mtgp_gpu_plan_t *plan[2] = {nullptr, nullptr};
    bool used[2] = {false, false};  // the batch has requests of the pool
    std::vector<Req> reqs;  // the batch (owned by the worker while busy)
    bool busy = false;      // holds a batch: handed over, launching or on the GPU
    bool assigned = false;  // handed over, not yet taken by the worker
    bool planning = false;  // handed over and not yet launched
    uint64_t seq = 0;       // number of the batch it holds (server-wide, from 1)
    uint64_t launched = 0;  // number of its latest batch whose launch is done (or failed)
    uint64_t retired = 0;   // number of its latest retired batch
    std::vector<uint64_t> deps[2];  // per pool, tags of the batches it must follow on the GPU
    uint64_t block = 0, block_bytes = 0;  // the batch's arena block
    bool has_block = false;               // placed in the arena
    std::vector<double> lat;              // latencies, computed before the retire
    std::thread th;         // the slot's worker
    std::condition_variable cv;
};

// A batch's tag for the streams' order: its number and its slot.
inline uint64_t batchTag(uint64_t seq, size_t slot) { return (seq << 8) | slot; }

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
    uint64_t next_place = 1;  // number of the batch whose turn it is to take arena space
    // arena bytes of admitted batches not yet placed, and of results kept in
    // the arena (counted from admission: they outlive their batch's block):
    // admission keeps ahead <= arena size - kept, so every batch admitted
    // fits in the arena once the batches on the GPU are done, and a request
    // that does not stays pending (and cancellable)
    uint64_t ahead = 0, kept_bytes = 0;
    uint64_t budget = 0;  // the arena's size
    uint64_t pending_bytes = 0;  // output bytes of the pending requests (rounded)
    std::vector<uint64_t> failed;  // numbers of batches that failed to launch (rare)
    // set when admission may take more: a submission, a retired batch or
    // released space since the scheduler's last admission pass
    bool dirty = false;
    bool sched_waiting = false;  // the scheduler sleeps on cv (a submission wakes it)
    std::mutex mu;
    // cv: the scheduler; cv_done: waiters for results; cv_turn: workers
    // waiting for their arena turn, space or an earlier batch's launch
    std::condition_variable cv, cv_done, cv_turn;
    std::deque<Req> pending;
    std::vector<char> mark[2];  // admission scratch per stream
    mtgp::StreamOrder order;
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
    int makeReq(int pool, uint32_t stream, int kind, uint64_t skip, uint64_t count, void *dst,
                bool keep, Req *r) const;
    void pushLocked(Req &r);

    void loop();
    void work(Slot &sl);
    int planBatch(Slot &sl, double *plan_s);
    int launchBatch(Slot &sl);
    int orderBatch(Slot &sl, std::unique_lock<std::mutex> &lk, int rc);
    bool placeNow(Slot &sl);
    void retireBatch(Slot &sl, int st);
};

// Refill the slot's plans with the batch (offsets relative to its block).
int mtgp_server::planBatch(Slot &sl, double *plan_s) {
    std::vector<mtgp_work_item_t> items[2];
    for (const Req &r : sl.reqs) {
        mtgp_work_item_t it{};
        it.stream = r.stream;
        it.kind = r.kind;
        it.count = r.count;
        it.out_offset = r.off;
        it.skip = r.skip;
        items[r.pool].push_back(it);
    }
    const Clock::time_point tp = Clock::now();
    int rc = MTGP_OK;
    for (int p = 0; p < 2 && !rc; p++) {
        const int n = (int)items[p].size();
        sl.used[p] = n > 0;
        if (!n) continue;
        if (!sl.plan[p]) {
            rc = p == 0 ? mtgp32_gpu_pool_plan(p32, items[p].data(), n, &sl.plan[p])
                        : mtgp64_gpu_pool_plan(p64, items[p].data(), n, &sl.plan[p]);
        } else {
            rc = p == 0 ? mtgp32_gpu_pool_replan(p32, items[p].data(), n, sl.plan[p])
                        : mtgp64_gpu_pool_replan(p64, items[p].data(), n, sl.plan[p]);
        }
    }
    *plan_s += std::chrono::duration<double>(Clock::now() - tp).count();
    return rc;
}

// Place a batch's block now if it is its turn and the arena has room (with
// the lock held; the scheduler tries it at admission, so that a batch whose
// planning is slow does not hold back the placement of the next ones).
bool mtgp_server::placeNow(Slot &sl) {
    if (sl.has_block || next_place != sl.seq || !arena.alloc(sl.block_bytes, &sl.block))
        return false;
    sl.has_block = true;
    next_place++;
    ahead -= sl.block_bytes;
    cv_turn.notify_all();
    return true;
}

// Take the batch's arena block in admission order (waiting for space) unless
// it was placed at admission, then order its CUDA stream after the batches
// that hold its streams (waiting for their launches).  With rc set (planning
// failed) only the turn is taken.  Called and returns with the lock held.
int mtgp_server::orderBatch(Slot &sl, std::unique_lock<std::mutex> &lk, int rc) {
    if (!sl.has_block) {
        cv_turn.wait(lk, [&] {
            if (stop.load()) return true;
            if (next_place != sl.seq) return false;
            return rc != MTGP_OK || placeNow(sl);
        });
        if (!sl.has_block) {  // planning failed, or stopping
            if (next_place == sl.seq) {
                next_place++;
                ahead -= sl.block_bytes;
                cv_turn.notify_all();
            }
            if (!rc) rc = mtgp::recordError(MTGP_ERR_BUSY, "stopping");
        }
    }
    if (!rc)
        for (Req &r : sl.reqs) r.off += sl.block;
    for (int p = 0; p < 2; p++)
        for (uint64_t tag : sl.deps[p]) {
            Slot &x = *slots[tag & 0xff];
            const uint64_t b = tag >> 8;
            cv_turn.wait(lk, [&] { return x.launched >= b || x.retired >= b || stop.load(); });
            if (rc) continue;
            if (std::find(failed.begin(), failed.end(), b) != failed.end()) {
                rc = mtgp::recordError(MTGP_ERR_CUDA, "an earlier batch of the same streams failed");
            } else if (x.retired < b) {
                // x cannot record dep_ev again before it retires b, which needs the lock
                cudaError_t e = cudaStreamWaitEvent(sl.cs[p], x.dep_ev[p], 0);
                if (e != cudaSuccess) rc = mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
            }
        }
    return rc;
}

int mtgp_server::launchBatch(Slot &sl) {
    cudaError_t e = cudaSuccess;
    for (int p = 0; p < 2; p++) {
        if (!sl.used[p]) continue;
        int rc = mtgp_gpu_plan_launch(sl.plan[p], d_arena + sl.block, sl.cs[p]);
        if (rc) return rc;
        e = cudaEventRecord(sl.dep_ev[p], sl.cs[p]);
        if (e != cudaSuccess) return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    }
    for (const Req &r : sl.reqs) {
        if (!r.dst || !r.bytes) continue;
        e = cudaMemcpyAsync(r.dst, d_arena + r.off, r.bytes, cudaMemcpyDefault, sl.cs[r.pool]);
        if (e != cudaSuccess) return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    }
    if (sl.used[1]) {
        e = cudaEventRecord(sl.join, sl.cs[1]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sl.cs[0], sl.join, 0);
        if (e != cudaSuccess) return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    }
    e = cudaEventRecord(sl.ev, sl.cs[0]);
    if (e != cudaSuccess) return mtgp::recordError(MTGP_ERR_CUDA, cudaGetErrorString(e));
    return MTGP_OK;
}

void mtgp_server::loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    std::vector<Req> take;
    while (!stop.load()) {
        bool progressed = false;
        size_t fi = slots.size();
        for (size_t k = 0; k < slots.size(); k++)
            if (!slots[k]->busy) {
                fi = k;
                break;
            }
        if (fi < slots.size() && dirty && !pending.empty() &&
            (nplanning == 0 || pending.size() >= (size_t)std::max(1, max_batch / 4))) {
            dirty = false;
            const Clock::time_point ta = Clock::now();
            Slot *fs = slots[fi].get();
            auto live = [this](uint64_t tag) {
                const Slot &x = *slots[tag & 0xff];
                return x.seq == (tag >> 8) && x.retired < x.seq;
            };
            // A stream with a batch in flight joins the new one (which the
            // GPU then runs after it) only under a backlog; otherwise it
            // waits, so that batches of a light load share no stream and
            // run side by side on the GPU instead of one after another.
            const bool pipe = pending.size() >= (size_t)std::max(1, max_batch / 4);
            // (Taking all that waits under a backlog locks a steady load near
            // capacity into batches whose formation and GPU time double the
            // latency.)
            const int cap = mtgp::batchCap(pending.size(), max_batch, pipe);
            fs->block_bytes = mtgp::admitBatch(
                pending, mark, cap, kJumpSkip, arena.size() - kept_bytes - ahead,
                mtgp::batchBytes(pending_bytes, arena.size()),
                [&](const Req &r) {
                    const uint64_t l = order.latest(r);
                    return !pipe && l && live(l);
                },
                &take, 4 * (size_t)max_batch);
            pending_bytes -= fs->block_bytes;
            if (!take.empty()) {
                const uint64_t seq = ++batches;
                // the batches still in flight that hold some of its streams
                order.order(take, batchTag(seq, fi), live, fs->deps);
                fs->reqs.swap(take);
                fs->seq = seq;
                ahead += fs->block_bytes;
                placeNow(*fs);
                for (const Req &r : fs->reqs)
                    if (r.keep) kept_bytes += Arena::round(r.bytes);
                fs->busy = fs->assigned = fs->planning = true;
                nplanning++;
                fs->cv.notify_one();
                dirty = true;  // another free slot may take more
                progressed = true;
            }
            prof[0] += std::chrono::duration<double>(Clock::now() - ta).count();
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
        // plan, take the arena block and the order on the GPU, launch, then
        // wait for the batch: a short spin, so that the retire follows a
        // short batch closely, then a blocking wait (the event is a
        // blocking-sync one), so that long batches hold no core
        const Clock::time_point tl = Clock::now();
        double plan_s = 0;
        int rc = planBatch(sl, &plan_s);
        for (int p = 0; p < 2 && !rc; p++)  // what needs no window nor output space
            if (sl.used[p]) rc = mtgp::planPrepare(sl.plan[p], sl.cs[p]);
        lk.lock();
        rc = orderBatch(sl, lk, rc);
        lk.unlock();
        if (!rc) rc = launchBatch(sl);
        // work already queued for this batch must end before its arena block
        // is handed to another batch
        if (rc) {
            cudaStreamSynchronize(sl.cs[0]);
            cudaStreamSynchronize(sl.cs[1]);
        }
        const Clock::time_point tw = Clock::now();
        lk.lock();
        sl.launched = sl.seq;
        if (rc) failed.push_back(sl.seq);
        cv_turn.notify_all();
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
        const int st = rc ? rc : q == cudaSuccess ? MTGP_OK : MTGP_ERR_CUDA;
        const Clock::time_point now = Clock::now();
        sl.lat.resize(sl.reqs.size());
        for (size_t k = 0; k < sl.reqs.size(); k++)
            sl.lat[k] = st ? 0 : std::chrono::duration<double>(now - sl.reqs[k].t_submit).count();
        lk.lock();
        prof[1] += std::chrono::duration<double>(tw - tl).count();
        prof[4] += plan_s;
        retireBatch(sl, st);
        prof[2] += std::chrono::duration<double>(Clock::now() - now).count();
    }
}

// With the lock held: record the batch's latencies and statuses, keep the
// results that stay in the arena and return the rest of its block.
void mtgp_server::retireBatch(Slot &sl, int st) {
    uint64_t at = sl.block;  // start of the block's part not yet returned
    for (size_t k = 0; k < sl.reqs.size(); k++) {
        const Req &r = sl.reqs[k];
        latency[r.ticket - 1] = sl.lat[k];
        status[r.ticket - 1] = st;
        if (r.keep && st) kept_bytes -= Arena::round(r.bytes);  // nothing to keep
        if (!st && r.keep && r.bytes) {
            kept[r.ticket] = {r.off, r.bytes};
            if (r.off > at) arena.release(at, r.off - at);
            at = r.off + Arena::round(r.bytes);
        }
        completed++;
        if (!st) bytes_done += r.bytes;
    }
    if (sl.has_block) {
        const uint64_t end = sl.block + mtgp::Arena::round(sl.block_bytes);
        if (end > at) arena.release(at, end - at);
    }
    sl.has_block = false;
    sl.reqs.clear();
    sl.retired = sl.seq;
    sl.busy = false;
    dirty = true;
    cv_turn.notify_all();
    cv.notify_one();
    cv_done.notify_all();
}

extern "C" {

int mtgp_server_create(mtgp_server_t **out, mtgp32_gpu_pool_t *p32, mtgp64_gpu_pool_t *p64,
                       uint64_t budget_bytes, int slots, int max_batch) {
    if (!out || (!p32 && !p64) || budget_bytes < 256 || slots < 1 || slots > 256 ||
        max_batch < 1)
        return mtgp::recordError(MTGP_ERR_INVALID, "bad server arguments");
    *out = nullptr;
    mtgp_server *s = new (std::nothrow) mtgp_server();
    if (!s) return mtgp::recordError(MTGP_ERR_ALLOC, "server allocation");
    s->p32 = p32;
    s->p64 = p64;
    s->nstreams[0] = p32 ? mtgp32_gpu_pool_size(p32) : 0;
    s->nstreams[1] = p64 ? mtgp64_gpu_pool_size(p64) : 0;
    s->mark[0].assign(s->nstreams[0], mtgp::kStreamFree);
    s->mark[1].assign(s->nstreams[1], mtgp::kStreamFree);
    s->order.init(s->nstreams[0], s->nstreams[1]);
    s->max_batch = max_batch;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = mtgp::devMalloc(&s->d_arena, budget_bytes);
    if (e != cudaSuccess) {
        delete s;
        return mtgp::recordError(MTGP_ERR_ALLOC, cudaGetErrorString(e));
    }
    s->arena.init(budget_bytes);
    s->budget = budget_bytes;
    for (int k = 0; k < slots; k++) {
        s->slots.emplace_back(new (std::nothrow) Slot());
        Slot *sl = s->slots.back().get();
        if (!sl) {
            s->slots.pop_back();
            e = cudaErrorMemoryAllocation;
            break;
        }
        for (int p = 0; p < 2; p++) {
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl->cs[p], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl->dep_ev[p], cudaEventDisableTiming);
        }
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming | cudaEventBlockingSync);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl->join, cudaEventDisableTiming);
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
    if (!ticket) return mtgp::recordError(MTGP_ERR_INVALID, "null ticket");
    Req r;
    const int rc = makeReq(pool, stream, kind, skip, count, dst, keep, &r);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(mu);
    pushLocked(r);
    *ticket = r.ticket;
    return MTGP_OK;
}

// A request checked and filled in, except its ticket (no lock: it reads only
// what the server's creation fixed).
int mtgp_server::makeReq(int pool, uint32_t stream, int kind, uint64_t skip, uint64_t count,
                         void *dst, bool keep, Req *r) const {
    if (pool < 0 || pool > 1 || stream >= (uint32_t)nstreams[pool])
        return mtgp::recordError(MTGP_ERR_INVALID, "no such pool or stream");
    if (kind < -1 || kind > 4) return mtgp::recordError(MTGP_ERR_INVALID, "unknown output kind");
    const uint64_t esz = pool == 0 ? 4u : 8u;
    if (kind >= 0 && count > ~uint64_t(0) / esz)
        return mtgp::recordError(MTGP_ERR_BUDGET, "request larger than the device budget");
    const uint64_t bytes = kind < 0 ? 0 : count * esz;
    if (mtgp::Arena::round(bytes) > budget)
        return mtgp::recordError(MTGP_ERR_BUDGET, "request larger than the device budget");
    *r = Req{};
    r->pool = pool;
    r->stream = stream;
    r->kind = kind;
    r->skip = skip;
    r->count = count;
    r->bytes = bytes;
    r->dst = dst;
    r->keep = keep && !dst;
    r->t_submit = Clock::now();
    return MTGP_OK;
}

// Queue a request (mu held): its ticket, its pending result slots; the
// scheduler is woken only when it sleeps, so a burst of submissions costs no
// wake-up each.
void mtgp_server::pushLocked(Req &r) {
    r.ticket = ++submitted;
    latency.push_back(-1.0);
    status.push_back(1);
    pending.push_back(r);
    pending_bytes += Arena::round(r.bytes);
    dirty = true;
    if (sched_waiting) cv.notify_one();
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
    s->kept_bytes -= mtgp::Arena::round(it->second.second);
    s->kept.erase(it);
    s->dirty = true;
    s->cv.notify_one();
    s->cv_turn.notify_all();  // a batch may wait for this space
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
        s->pending_bytes -= mtgp::Arena::round(it->bytes);
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
    std::vector<Req> due_now;
    for (int k = 0; k < n;) {
        const Clock::time_point at = due(k);
        while (Clock::now() < at) {
            const auto left = at - Clock::now();
            if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left / 2);
        }
        // the requests already due (at most 256), made outside the lock and
        // queued under one; then the lock is left to the scheduler for a
        // moment, so that admission starts while a burst is still queued
        const Clock::time_point now = Clock::now();
        const int k0 = k;
        due_now.clear();
        int rc = MTGP_OK;
        do {
            const mtgp_request_t &r = reqs[k];
            Req q;
            rc = s->makeReq(r.pool, r.stream, r.kind, r.skip, r.count, r.dst, false, &q);
            if (rc) break;
            due_now.push_back(q);
            k++;
        } while (k < n && k - k0 < 256 && due(k) <= now);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Req &q : due_now) s->pushLocked(q);
        }
        if (rc) return rc;
        std::this_thread::yield();
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
        s->cv_turn.notify_all();
        for (auto &sp : s->slots) sp->cv.notify_all();
    }
    if (s->th.joinable()) s->th.join();
    for (auto &sp : s->slots)
        if (sp->th.joinable()) sp->th.join();
    for (auto &sp : s->slots) {
        Slot &sl = *sp;
        for (int p = 0; p < 2; p++)
            if (sl.cs[p]) cudaStreamSynchronize(sl.cs[p]);
        for (int p = 0; p < 2; p++) mtgp_gpu_plan_free(sl.plan[p]);
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.join) cudaEventDestroy(sl.join);
        for (int p = 0; p < 2; p++) {
            if (sl.dep_ev[p]) cudaEventDestroy(sl.dep_ev[p]);
            if (sl.cs[p]) cudaStreamDestroy(sl.cs[p]);
        }
    }
    cudaFree(s->d_arena);
    delete s;
}

}  // extern "C"
