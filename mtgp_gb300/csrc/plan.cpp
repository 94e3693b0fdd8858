// plan.cpp -- batched plans: the planner driver (items -> tasks, jump
// polynomials, jumps made ahead of the launch, the device blob), their
// launch, and the plan entry points of the C ABI.
#include "host_internal.h"

namespace mtgp {
namespace host {

// A jump polynomial X^steps mod chi_pidx computed on the GPU at launch.
struct GpuJob {
    int pidx;
    uint64_t steps;
    int32_t slot;
    const uint32_t *tab;  // the device tables of parameter set pidx
};

template <class T>
int makePlan(Pool<T> &P, const mtgp_work_item_t *items, int nitems, mtgp_gpu_plan **out,
             int force_core, int64_t force_chunk) {
    using W = typename T::W;
    if (!out) return setErr(MTGP_ERR_INVALID, "null plan pointer");
    if (*out && (*out)->pool != &P) return setErr(MTGP_ERR_INVALID, "plan belongs to another pool");
    PlanOptions o;
    o.nstreams = P.count;
    o.word_bytes = sizeof(W);
    o.can_jump = planJumps(P);
    o.jump_min = jumpMinSkip(P);
    o.max_gen_skip = kMaxGenSkip;
    o.chunk_tune = force_chunk ? force_chunk : P.tune.split_chunk;
    // Whether the generated values mix kinds (a generated skip counts as kind
    // -1): the same rule as planCore's mode, decided up front because the
    // chunk length depends on the core's resident CTAs.  Plans of mixed kinds
    // take the one-word core unless a core is forced (the autotuner's
    // candidates): the 32-bit two- and four-word kernels run mixed kinds too
    // (each kind's loop out of line), 5-7 % faster on long steady batches,
    // but serving batches of many short requests had longer tails on them
    // (p99 at 0.9 load 5-7 ms against 2.5 ms); the 64-bit two-word kernel has
    // one kind per launch.
    int kinds = -3;
    auto addKind = [&kinds](int k) { kinds = (kinds == -3 || kinds == k) ? k : -2; };
    auto jumped = [&o](uint64_t v) { return o.can_jump && v >= o.jump_min; };
    for (int k = 0; k < nitems && items; k++) {
        const mtgp_work_item_t &it = items[k];
        if (it.kind < 0) {
            const uint64_t adv = it.skip + it.count;
            if (adv && !jumped(adv)) addKind(-1);
        } else {
            if (it.skip && !jumped(it.skip)) addKind(-1);
            if (it.count) addKind(it.kind);
        }
    }
    int core = force_core ? force_core : kinds == -2 ? 1 : P.tune.core;
    // 64-bit cores: two words per thread (knob 2 or 4) or one; the two-word
    // kernel has no jump code, so plans with in-kernel jumps (jump_parts =
    // -1) take the one-word core
    if (T::kBits == 64) core = (core == 1 || P.tune.jump_parts < 0) ? 1 : 2;
    // where the kernel has no jump code (the exponents without the in-kernel
    // jump, the 64-bit two-word core) every jumped start is made ahead of
    // the launch, from one polynomial (a run start and a chunk offset
    // combined)
    const bool kernel_jumps = T::splits(P.sh.mexp) && (T::kBits == 32 || core == 1);
    // with jumps made ahead of the launch, the kernel without the jump code
    o.resident = o.can_jump ? T::resident(P.sh.mexp, P.tune.jump_parts < 0, core) : 1;
    // scratch reused by every plan made on this thread
    static thread_local PlanResult R;
    std::string msg;
    int rc = planCore(items, nitems, o, &R, &msg);
    if (rc) return setErr(rc, "%s", msg.c_str());
    const uint64_t out_bytes = R.out_bytes;
    const int64_t chunk = R.chunk;
    const bool cut = chunk > 0;
    const int mode = R.mode;
    std::vector<int32_t> &stage_streams = R.stage_streams;
    // the plan's jump polynomials: X^steps mod chi for (parameter set, steps)
    const size_t pw = (size_t)P.polyWords();
    std::map<std::pair<int, uint64_t>, int> poly_at;
    std::vector<uint32_t> polys;  // computed here, in index order
    // A requested skip (a run start) that the host has not cached and would
    // need a product for (two or more set bits) is computed on the GPU at
    // launch (GpuJob): arbitrary offsets then cost the host nothing.  Chunk
    // offsets recur from plan to plan and stay on the host, cached.  Until
    // the indices are final, GPU polynomials carry kGpuSlot + job number.
    constexpr int32_t kGpuSlot = 1 << 29;
    std::vector<GpuJob> gjobs;
    auto polyIndex = [&](int pidx, uint64_t steps, int32_t *idx, bool gpu_ok) -> int {
        // the plan's own map first (most tasks of a plan share their
        // polynomials), the pool's caches under its lock only on a miss
        auto hit = poly_at.find({pidx, steps});
        if (hit == poly_at.end()) {
            std::lock_guard<std::recursive_mutex> lk(P.cache_mu);
            int slot;
            if (gpu_ok && P.jcache.find({pidx, steps}) == P.jcache.end() &&
                __builtin_popcountll(steps) >= 2) {
                const uint32_t *t = nullptr;
                int rc2 = P.gpuPowTables(pidx, &t);  // made now, never during a launch
                if (rc2) return rc2;
                slot = kGpuSlot + (int)gjobs.size();
                gjobs.push_back(GpuJob{pidx, steps, slot, t});
            } else {
                const gf2::Poly *p = nullptr;
                int rc2 = P.jumpPoly(pidx, steps, &p);
                if (rc2) return rc2;
                slot = (int)(polys.size() / pw);
                const std::vector<uint32_t> w = gf2::toWords32(*p, (int)pw);
                polys.insert(polys.end(), w.begin(), w.end());
            }
            hit = poly_at.emplace(std::make_pair(pidx, steps), slot).first;
        }
        *idx = hit->second;
        return MTGP_OK;
    };
    // Where neither the kernel nor jumps ahead of the launch (jump_parts < 0)
    // can apply a run start and a chunk offset one after the other, the two
    // make one polynomial.
    const bool combined = !kernel_jumps && P.tune.jump_parts < 0;
    // every parameter set that jumps gets its tables in one batch, and the
    // chunk offsets not yet cached (with the run start where the two make
    // one polynomial) go to the GPU together, for later plans
    {
        std::vector<int> sets;
        std::vector<std::pair<int, uint64_t>> offs;
        for (const PlanTask &pt : R.tasks) {
            if (!pt.run && !pt.off) continue;
            const int k = P.hpidx[pt.stream];
            if (std::find(sets.begin(), sets.end(), k) == sets.end()) sets.push_back(k);
            const uint64_t e = pt.run && combined ? pt.run + pt.off : pt.off;
            if (pt.off && __builtin_popcountll(e) >= 2) offs.emplace_back(k, e);
        }
        {
            std::lock_guard<std::recursive_mutex> lk(P.cache_mu);
            rc = P.prepare(sets);
        }
        if (!rc) rc = P.startFill(offs);
        if (rc) return rc;
    }
    std::vector<BatchTask> tasks(R.tasks.size());
    for (size_t q = 0; q < R.tasks.size(); q++) {
        const PlanTask &pt = R.tasks[q];
        BatchTask &t = tasks[q];
        t = BatchTask{};
        t.stream = pt.stream;
        t.first = (int32_t)pt.first;
        t.nitems = (int32_t)pt.n;
        t.pidx = P.hpidx[pt.stream];
        t.j0 = t.j1 = -1;
        t.wb = pt.wb;
        // X^run then X^off: the run starts (a requested skip) and the chunk
        // offsets (shared by every long request) are each few, so few
        // distinct polynomials are needed
        if (pt.run && pt.off && combined) {
            rc = polyIndex(t.pidx, pt.run + pt.off, &t.j0, true);
        } else if (pt.run && pt.off) {
            rc = polyIndex(t.pidx, pt.run, &t.j0, true);
            if (!rc) rc = polyIndex(t.pidx, pt.off, &t.j1, true);
        } else if (pt.run || pt.off) {
            rc = polyIndex(t.pidx, pt.run | pt.off, &t.j0, true);
        }
        if (rc) return rc;
    }
    std::vector<BatchItem> bitems(R.segs.size());
    for (size_t q = 0; q < R.segs.size(); q++) {
        bitems[q].out_off = R.segs[q].out_off;
        bitems[q].count = R.segs[q].count;
        bitems[q].kind = R.segs[q].kind;
        bitems[q].pad_ = 0;
    }
    // final indices of the GPU-computed polynomials: after the host's,
    // grouped by parameter set so that each group is one launch
    const int nhost = (int)(polys.size() / pw);
    std::stable_sort(gjobs.begin(), gjobs.end(),
                     [](const GpuJob &a, const GpuJob &b) { return a.pidx < b.pidx; });
    std::vector<int32_t> remap(gjobs.size());
    std::vector<uint64_t> job_steps(gjobs.size());
    for (size_t q = 0; q < gjobs.size(); q++) {
        remap[(size_t)(gjobs[q].slot - kGpuSlot)] = nhost + (int32_t)q;
        job_steps[q] = gjobs[q].steps;
    }
    static thread_local PowSchedule sch;
    powSchedule(job_steps.data(), (int)job_steps.size(), job_steps.empty() ? 1 : P.powWidth(),
                sch);
    for (BatchTask &t : tasks) {
        if (t.j0 >= kGpuSlot) t.j0 = remap[(size_t)(t.j0 - kGpuSlot)];
        if (t.j1 >= kGpuSlot) t.j1 = remap[(size_t)(t.j1 - kGpuSlot)];
    }
    const size_t npolys = (size_t)nhost + gjobs.size();
    // A task that starts with one jump takes its window from a slot made
    // ahead of the launch by jump parts (jumpParts() CTAs per jump, all
    // SMs at once), so no jump runs inside the persistent kernel; a chain of
    // two (a run start, then a chunk offset) still jumps inside it.
    // A task that jumps twice (a run start, then a chunk offset) is jumped
    // ahead in two launches: the run start once per run, from the stream's
    // window into a middle slot (after the tasks' slots), with the single
    // jumps; then each chunk offset from its run's middle slot (their source
    // offsets are relative to the slots).
    static thread_local std::vector<JumpPart> jparts;
    static thread_local std::vector<JumpPart> jparts_b;
    jparts.clear();
    jparts_b.clear();
    int npre = 0, nmid = 0;
    if (P.tune.jump_parts >= 0 && npolys > 0) {
        const int tch = T::jumpChunks(P.sh.mexp, (int)pw);
        const int parts = jumpParts(P.tune, tch);
        auto addParts = [&](std::vector<JumpPart> &v, uint64_t src, int32_t poly, int32_t dst,
                            int32_t pidx) {
            for (int q = 0; q < parts; q++) {
                JumpPart d{};
                d.src = src;
                d.poly = poly;
                d.dst = dst;
                d.pidx = pidx;
                d.ch0 = (int16_t)partChunk(q, tch, parts);
                d.ch1 = (int16_t)partChunk(q + 1, tch, parts);
                v.push_back(d);
            }
        };
        for (BatchTask &t : tasks)
            if (t.j0 >= 0) t.pre = ++npre;
        std::map<std::pair<int32_t, uint64_t>, int32_t> mid;  // (stream, run) -> middle slot
        for (size_t q = 0; q < tasks.size(); q++) {
            BatchTask &t = tasks[q];
            if (t.j0 < 0) continue;
            const uint64_t win = (uint64_t)t.stream * (uint64_t)P.stride;
            if (t.j1 < 0) {
                addParts(jparts, win, t.j0, t.pre - 1, t.pidx);
            } else {
                auto it = mid.find({t.stream, R.tasks[q].run});
                if (it == mid.end()) {
                    it = mid.emplace(std::make_pair(t.stream, R.tasks[q].run), npre + nmid++).first;
                    addParts(jparts, win, t.j0, it->second, t.pidx);
                }
                addParts(jparts_b, (uint64_t)it->second * (uint64_t)P.stride, t.j1, t.pre - 1,
                         t.pidx);
            }
            t.j0 = t.j1 = -1;
        }
    }
    // jump_overlap: the tasks that start from a pre-jumped window go last,
    // each group in its longest-first order (a second launch runs them)
    int nmain = (int)tasks.size();
    if (P.tune.jump_overlap > 0 && npre > 0) {
        std::stable_partition(tasks.begin(), tasks.end(),
                              [](const BatchTask &t) { return t.pre == 0; });
        nmain = 0;
        while (nmain < (int)tasks.size() && tasks[(size_t)nmain].pre == 0) nmain++;
    }
    bool split = false;  // the kernel variant with the jump code
    for (const BatchTask &t : tasks) split = split || t.j0 >= 0;
    // reuse the caller's plan (replan) when given: its device buffers are
    // kept and only grown, so a server can refill plans without freeing
    // device memory (cudaFree would wait for every batch in flight)
    mtgp_gpu_plan *pl = *out;
    const bool fresh = (pl == nullptr);
    if (fresh) {
        pl = new (std::nothrow) mtgp_gpu_plan();
        if (!pl) return setErr(MTGP_ERR_ALLOC, "plan allocation");
    } else if (pl->exec) {
        cudaGraphExecDestroy(pl->exec);
        pl->exec = nullptr;
        pl->graph_out = nullptr;
    }
    pl->bits = T::kBits;
    pl->pool = &P;
    pl->ntasks = (int)tasks.size();
    pl->mode = mode;
    pl->out_bytes = out_bytes;
    pl->grid = (int)P.tune.batch_grid;
    pl->split = split;
    pl->core = core;
    pl->chunk = cut ? chunk : 0;
    pl->nstage = (int)stage_streams.size();
    pl->npre = npre;
    pl->nmid = nmid;
    pl->nparts = (int)jparts.size();
    pl->nparts_b = (int)jparts_b.size();
    pl->overlap = nmain < (int)tasks.size();
    pl->nmain = nmain;
    auto align = [](size_t n) { return (n + 255) & ~size_t(255); };
    const size_t off_items = align(sizeof(BatchTask) * tasks.size());
    const size_t off_polys = off_items + align(sizeof(BatchItem) * bitems.size());
    const size_t off_ops = off_polys + align(sizeof(uint32_t) * pw * npolys);
    const size_t off_parts = off_ops + align(sizeof(PowOp) * (size_t)sch.steps());
    const size_t off_ss =
        off_parts + align(sizeof(JumpPart) * (jparts.size() + jparts_b.size()));
    const size_t bytes = off_ss + sizeof(int32_t) * stage_streams.size();
    cudaError_t e = cudaSuccess;
    if (!pl->d_counter) e = devMalloc(&pl->d_counter, 2 * sizeof(unsigned));
    if (e == cudaSuccess && pl->overlap && !pl->side) {
        e = cudaStreamCreateWithFlags(&pl->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->join, cudaEventDisableTiming);
    }
    // Buffers only grow, to twice what is needed, and a buffer replaced by a
    // larger one is freed with the plan: freeing it now (cudaFree,
    // cudaFreeHost) would wait for every launch in flight on the device, and
    // an earlier launch of this plan may still read it.
    auto growDev = [pl](auto **buf, size_t *cap, size_t need) -> cudaError_t {
        if (need <= *cap) return cudaSuccess;
        if (*buf) pl->retired_dev.push_back(*buf);
        *buf = nullptr;
        *cap = 0;
        const size_t n = std::max<size_t>(2 * need, 4096);
        cudaError_t err = devMallocRaw(reinterpret_cast<void **>(buf), n);
        if (err == cudaSuccess) *cap = n;
        return err;
    };
    if (e == cudaSuccess) e = growDev(&pl->d_blob, &pl->cap_d, bytes);
    if (e == cudaSuccess && bytes > pl->cap_h) {
        if (pl->h_blob) pl->retired_host.push_back(pl->h_blob);
        pl->h_blob = nullptr;
        pl->cap_h = 0;
        const size_t n = std::max<size_t>(2 * bytes, 4096);
        e = hostAlloc(&pl->h_blob, n);
        if (e == cudaSuccess) pl->cap_h = n;
    }
    if (e == cudaSuccess) {
        size_t cap = pl->cap_pscratch * sizeof(uint32_t);
        e = growDev(&pl->d_pscratch, &cap, sizeof(uint32_t) * (size_t)sch.nscratch * pw);
        pl->cap_pscratch = cap / sizeof(uint32_t);
    }
    if (e == cudaSuccess && pl->nstage)
        e = growDev(&pl->d_stage, &pl->cap_stage, sizeof(W) * (size_t)P.stride * pl->nstage);
    if (e == cudaSuccess && pl->npre) {
        const size_t before = pl->cap_prewin;
        e = growDev(&pl->d_prewin, &pl->cap_prewin,
                    sizeof(W) * (size_t)P.stride * (pl->npre + pl->nmid));
        if (pl->cap_prewin != before) pl->prewin_fresh = true;
    }
    if (e != cudaSuccess) {
        if (fresh) {
            delete pl;
        } else {  // a refilled plan that could not grow launches nothing
            pl->ntasks = 0;
            pl->nstage = 0;
            pl->npre = 0;
            pl->nmid = 0;
            pl->nparts = 0;
            pl->nparts_b = 0;
            pl->out_bytes = 0;
            pl->dirty = false;
        }
        return cudaErr(e, "plan buffers");
    }
    unsigned char *h = pl->h_blob;
    if (!tasks.empty()) std::memcpy(h, tasks.data(), sizeof(BatchTask) * tasks.size());
    if (!bitems.empty()) std::memcpy(h + off_items, bitems.data(), sizeof(BatchItem) * bitems.size());
    if (!polys.empty()) std::memcpy(h + off_polys, polys.data(), sizeof(uint32_t) * polys.size());
    pl->pow_levels.clear();
    if (sch.steps()) {  // GPU job q writes polynomial nhost + q
        static thread_local std::vector<PowOp> ops;
        uint32_t *dst = reinterpret_cast<uint32_t *>(pl->d_blob + off_polys) + (size_t)nhost * pw;
        std::vector<const uint32_t *> tabs(gjobs.size());
        for (size_t q = 0; q < gjobs.size(); q++) tabs[q] = gjobs[q].tab;
        P.powOps(sch, [&tabs](int j) { return tabs[(size_t)j]; }, dst, pl->d_pscratch,
                 P.sh.mexp, ops);
        std::memcpy(h + off_ops, ops.data(), sizeof(PowOp) * ops.size());
        for (const auto &lev : sch.levels) pl->pow_levels.push_back((int)lev.size());
    }
    pl->d_powops = reinterpret_cast<const PowOp *>(pl->d_blob + off_ops);
    if (!jparts.empty())
        std::memcpy(h + off_parts, jparts.data(), sizeof(JumpPart) * jparts.size());
    if (!jparts_b.empty())
        std::memcpy(h + off_parts + sizeof(JumpPart) * jparts.size(), jparts_b.data(),
                    sizeof(JumpPart) * jparts_b.size());
    pl->d_parts = reinterpret_cast<const JumpPart *>(pl->d_blob + off_parts);
    if (!stage_streams.empty())
        std::memcpy(h + off_ss, stage_streams.data(), sizeof(int32_t) * stage_streams.size());
    pl->blob_bytes = bytes;
    pl->dirty = bytes > 0;
    pl->d_tasks = reinterpret_cast<const BatchTask *>(pl->d_blob);
    pl->d_items = reinterpret_cast<const BatchItem *>(pl->d_blob + off_items);
    pl->d_polys = reinterpret_cast<const uint32_t *>(pl->d_blob + off_polys);
    pl->d_stage_streams = reinterpret_cast<const int32_t *>(pl->d_blob + off_ss);
    *out = pl;
    return MTGP_OK;
}

// Zero a newly allocated pre-jumped window buffer, ordered before the next
// launch on s (afterwards the batched kernel zeroes each slot as it reads it).
int clearPrewin(mtgp_gpu_plan *pl, void *s) {
    if (!pl->prewin_fresh) return MTGP_OK;
    CK(cudaMemsetAsync(pl->d_prewin, 0, pl->cap_prewin, S(s)), "clear jumped windows");
    pl->prewin_fresh = false;
    return MTGP_OK;
}

// The plan's descriptors to the device, ordered before the next launch on s.
int uploadPlan(mtgp_gpu_plan *pl, void *s) {
    if (!pl->dirty) return MTGP_OK;
    CK(cudaMemcpyAsync(pl->d_blob, pl->h_blob, pl->blob_bytes, cudaMemcpyHostToDevice, S(s)),
       "upload plan");
    pl->dirty = false;
    pl->pow_ready = pl->pow_levels.empty();  // the upload overwrote the GPU-made polynomials
    return MTGP_OK;
}

// The plan's GPU-made jump polynomials (after the host-made ones in the
// blob), on s after the upload; they stay valid for later launches until
// the plan is refilled.
int powJobs(mtgp_gpu_plan *pl, int pw, int window, void *s) {
    if (pl->pow_ready) return MTGP_OK;
    size_t first = 0;
    for (int n : pl->pow_levels) {
        CK(launchPowOps(pl->d_powops + first, n, pl->d_pscratch, pw, S(s), window),
           "jump polynomials");
        first += (size_t)n;
    }
    pl->pow_ready = true;
    return MTGP_OK;
}

template <class T>
int launchPlan(mtgp_gpu_plan *pl, void *out, void *s) {
    Pool<T> &P = *static_cast<Pool<T> *>(pl->pool);
    if (pl->ntasks == 0) return MTGP_OK;
    if (pl->out_bytes && !out) return setErr(MTGP_ERR_INVALID, "null output pointer");
    int rc = uploadPlan(pl, s);
    if (!rc) rc = powJobs(pl, P.polyWords(), P.tune.poly_window, s);
    if (!rc) rc = clearPrewin(pl, s);
    if (rc) return rc;
    // with jump_overlap the jump parts and the tasks that wait for them go
    // to the side stream
    cudaStream_t js = pl->overlap ? pl->side : S(s);
    if (pl->overlap) {
        CK(cudaEventRecord(pl->fork, S(s)), "fork");
        CK(cudaStreamWaitEvent(pl->side, pl->fork, 0), "fork");
    }
    if (pl->nparts) {  // the start windows jumped ahead of the launch, into zeroed slots
        using W = typename T::W;
        W *pre = static_cast<W *>(pl->d_prewin);
        CK(T::parts(P.sh.mexp, P.d_params, P.d_states, pl->d_polys, P.polyWords(), pre, P.stride,
                    pl->d_parts, pl->nparts, js),
           "jumps ahead of the launch");
        if (pl->nparts_b) {  // chunk offsets from the run starts in the middle slots
            CK(T::parts(P.sh.mexp, P.d_params, pre, pl->d_polys, P.polyWords(), pre, P.stride,
                        pl->d_parts + pl->nparts, pl->nparts_b, js),
               "jumps ahead of the launch");
            CK(cudaMemsetAsync(pre + (size_t)pl->npre * P.stride, 0,
                               sizeof(W) * (size_t)P.stride * pl->nmid, js),
               "clear the middle slots");
        }
    }
    BatchLaunch b{};
    b.mexp = P.sh.mexp;
    b.mode = pl->mode;
    b.grid = pl->grid;
    b.nwords = P.polyWords();
    b.polys = pl->d_polys;
    b.split = pl->split;
    b.core = pl->core;
    b.tasks = pl->d_tasks;
    b.ntasks = pl->ntasks;
    b.items = pl->d_items;
    b.out = out;
    b.counter = pl->d_counter;
    b.stage = pl->d_stage;
    b.stage_streams = pl->d_stage_streams;
    b.nstage = pl->nstage;
    b.prewin = pl->d_prewin;
    cudaError_t e = cudaSuccess;
    if (pl->overlap) {
        BatchLaunch b2 = b;
        b2.tasks = pl->d_tasks + pl->nmain;
        b2.ntasks = pl->ntasks - pl->nmain;
        b2.counter = pl->d_counter + 1;
        b2.nstage = 0;
        b2.grid = 0;
        b.ntasks = pl->nmain;
        b.nstage = 0;
        e = T::batch(b2, P.d_params, P.d_states, pl->side);
        if (e == cudaSuccess) e = T::batch(b, P.d_params, P.d_states, S(s));
        if (e == cudaSuccess) e = cudaEventRecord(pl->join, pl->side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(S(s), pl->join, 0);
        if (e == cudaSuccess && pl->nstage)
            e = T::unstage(P.sh.mexp, P.d_states, pl->d_stage, pl->d_stage_streams, pl->nstage,
                           S(s));
    } else {
        e = T::batch(b, P.d_params, P.d_states, S(s));
    }
    if (e != cudaSuccess) {
        pl->prewin_fresh = pl->npre > 0;  // the slots may hold jump parts: zero them again
        return cudaErr(e, "batched launch");
    }
    return MTGP_OK;
}

int planLaunch(mtgp_gpu_plan *pl, void *out, void *s) {
    return pl->bits == 32 ? launchPlan<T32>(pl, out, s) : launchPlan<T64>(pl, out, s);
}


template int makePlan<T32>(Pool<T32> &, const mtgp_work_item_t *, int, mtgp_gpu_plan **, int,
                           int64_t);
template int makePlan<T64>(Pool<T64> &, const mtgp_work_item_t *, int, mtgp_gpu_plan **, int,
                           int64_t);
template int launchPlan<T32>(mtgp_gpu_plan *, void *, void *);
template int launchPlan<T64>(mtgp_gpu_plan *, void *, void *);

}  // namespace host

int planPrepare(mtgp_gpu_plan_t *pl, void *s) {
    if (!pl) return setErr(MTGP_ERR_INVALID, "null plan");
    int rc = uploadPlan(pl, s);
    if (!rc) {
        const int pw = pl->bits == 32 ? static_cast<Pool<T32> *>(pl->pool)->polyWords()
                                      : static_cast<Pool<T64> *>(pl->pool)->polyWords();
        const int win = pl->bits == 32 ? static_cast<Pool<T32> *>(pl->pool)->tune.poly_window
                                       : static_cast<Pool<T64> *>(pl->pool)->tune.poly_window;
        rc = powJobs(pl, pw, win, s);
    }
    if (!rc) rc = clearPrewin(pl, s);
    return rc;
}

}  // namespace mtgp

extern "C" {

int mtgp_gpu_plan_launch(mtgp_gpu_plan_t *pl, void *out, void *s) {
    if (!pl) return setErr(MTGP_ERR_INVALID, "null plan");
    return planLaunch(pl, out, s);
}

int mtgp_gpu_plan_graph_launch(mtgp_gpu_plan_t *pl, void *out, void *s) {
    if (!pl) return setErr(MTGP_ERR_INVALID, "null plan");
    if (!s) return setErr(MTGP_ERR_INVALID, "graph launch needs a non-default stream");
    if (!pl->exec || pl->graph_out != out) {
        if (pl->exec) {
            cudaGraphExecDestroy(pl->exec);
            pl->exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        // before the capture: replays reuse the descriptors and the GPU-made
        // jump polynomials
        int up = mtgp::planPrepare(pl, s);
        if (up) return up;
        CK(cudaStreamBeginCapture(S(s), cudaStreamCaptureModeThreadLocal), "begin capture");
        int rc = planLaunch(pl, out, s);
        cudaError_t e = cudaStreamEndCapture(S(s), &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cudaErr(e, "end capture");
        e = cudaGraphInstantiate(&pl->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cudaErr(e, "instantiate graph");
        pl->graph_out = out;
    }
    CK(cudaGraphLaunch(pl->exec, S(s)), "graph launch");
    return MTGP_OK;
}

uint64_t mtgp_gpu_plan_output_bytes(const mtgp_gpu_plan_t *pl) { return pl ? pl->out_bytes : 0; }

int mtgp_gpu_plan_info(const mtgp_gpu_plan_t *pl, int64_t *tasks, int64_t *chunk) {
    if (!pl) return setErr(MTGP_ERR_INVALID, "null plan");
    if (tasks) *tasks = pl->ntasks;
    if (chunk) *chunk = pl->chunk;
    return MTGP_OK;
}

int mtgp_gpu_plan_describe(const mtgp_gpu_plan_t *pl, int64_t *values, int n) {
    if (!pl || (n > 0 && !values)) return setErr(MTGP_ERR_INVALID, "null plan or values");
    const int64_t v[8] = {pl->ntasks, pl->chunk, pl->core, pl->grid,
                          pl->ntasks ? 1 + (pl->nstage > 0) + (pl->nparts > 0) +
                                           (pl->nparts_b > 0) +
                                           (pl->overlap && pl->nmain > 0)
                                     : 0,
                          pl->split ? 1 : 0, pl->npre, pl->overlap ? 1 : 0};
    for (int k = 0; k < n && k < 8; k++) values[k] = v[k];
    return MTGP_OK;
}

void mtgp_gpu_plan_free(mtgp_gpu_plan_t *pl) {
    if (!pl) return;
    cudaDeviceSynchronize();
    delete pl;
}

}  // extern "C"
