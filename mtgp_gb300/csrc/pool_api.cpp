// pool_api.cpp -- pools of device-resident streams and the autotuner:
// their entry points of the C ABI.
#include "host_internal.h"

namespace {

// Autotuner: build one plan per candidate configuration, time each on the
// caller's own items and output buffer (CUDA events on the caller's stream,
// median of `reps` launches after one warm-up), and keep the fastest.  The
// stream windows are restored from a snapshot before every launch, so every
// candidate does exactly the same work and the pool ends where it started.
// Candidates: generation core (32-bit: four words per thread in 64-thread
// CTAs with 128-bit stores, or one word per thread in 256-thread CTAs with
// 32-bit stores), split-chunk length for long requests (none, or 2^17 to
// 2^20 in steps of 2^17, with either core), and grid size (all resident
// CTAs, or 7/8, 3/4, 5/8, 1/2 of them).
template <class T>
int autotune(Pool<T> &P, const mtgp_work_item_t *items, int nitems, void *out, void *s,
             int reps, mtgp_gpu_plan **best, char *report, int cap) {
    using W = typename T::W;
    if (!best) return setErr(MTGP_ERR_INVALID, "null plan pointer");
    *best = nullptr;
    if (reps < 1) reps = 1;
    struct Cand {
        int core;
        int64_t chunk, grid;
        int overlap;
    };
    std::vector<Cand> cands;
    // 32-bit: four, two or one words per thread; 64-bit: two or one
    const int cores32[3] = {4, 2, 1}, cores64[2] = {2, 1};
    const int *cores = T::kBits == 32 ? cores32 : cores64;
    const int ncores = T::kBits == 32 ? 3 : 2;
    for (int c = 0; c < ncores; c++) cands.push_back({cores[c], -1, 0, 0});
    // chunk lengths: 1..8 times the shortest jumped piece (2^17 at MEXP
    // 11213 and 23209)
    const int64_t base = std::max<int64_t>(int64_t(1) << 17, (int64_t)jumpMinSkip(P));
    // (jump_overlap is left out: on the bench workload and the 128-set bank
    // it measured 1.3-2.7x slower, its jumped tasks being the longest ones)
    if (planJumps(P))
        for (int c = 0; c < ncores; c++)
            for (int64_t ch = base; ch <= 8 * base; ch += base)
                cands.push_back({cores[c], ch, 0, 0});
    const size_t sbytes = sizeof(W) * (size_t)P.stride * P.count;
    W *snap = nullptr;
    CK(devMalloc(&snap, sbytes), "devMalloc(autotune snapshot)");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const Tuning saved = P.tune;
    std::string rep;
    float best_ms = 0;
    int rc = MTGP_OK;
    cudaError_t ce = cudaMemcpyAsync(snap, P.d_states, sbytes, cudaMemcpyDeviceToDevice, S(s));
    if (ce != cudaSuccess) rc = cudaErr(ce, "autotune snapshot");
    // median of `reps` launches after one warm-up: a persistent launch's
    // length varies with the order its CTAs happen to take tasks in, and the
    // minimum would favour plans whose length varies most
    auto timeOne = [&](mtgp_gpu_plan *pl, float *ms) -> int {
        std::vector<float> ts;
        for (int r = 0; r <= reps; r++) {
            cudaError_t e = cudaMemcpyAsync(P.d_states, snap, sbytes, cudaMemcpyDeviceToDevice, S(s));
            if (e == cudaSuccess) e = cudaEventRecord(e0, S(s));
            if (e != cudaSuccess) return cudaErr(e, "autotune");
            int r2 = launchPlan<T>(pl, out, s);
            if (r2) return r2;
            e = cudaEventRecord(e1, S(s));
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float t = 0;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
            if (e != cudaSuccess) return cudaErr(e, "autotune timing");
            if (r > 0) ts.push_back(t);
        }
        std::sort(ts.begin(), ts.end());
        *ms = ts[ts.size() / 2];
        return MTGP_OK;
    };
    for (size_t k = 0; k < cands.size() && !rc; k++) {
        static const int kGridEighths[] = {8, 7, 6, 5, 4};  // of the resident CTAs
        for (int g = 0; g < 5 && !rc; g++) {
            P.tune.split_chunk = cands[k].chunk;
            P.tune.batch_grid = 0;
            P.tune.core = cands[k].core;
            P.tune.jump_overlap = cands[k].overlap;
            mtgp_gpu_plan *pl = nullptr;
            rc = makePlan(P, items, nitems, &pl);
            if (rc) break;
            if ((cands[k].chunk > 0 && pl->chunk == 0) ||       // nothing long enough to split
                (cands[k].overlap && !pl->overlap)) {           // nothing jumped ahead
                delete pl;
                break;
            }
            if (g > 0) {
                // fewer CTAs than resident: fewer share an SM's data pipe,
                // so each runs its tasks faster, which pays when the longest
                // tasks set the launch's length
                const int full = T::resident(P.sh.mexp, pl->split, pl->core);
                pl->grid = std::max(1, full * kGridEighths[g] / 8);
            }
            float ms = 0;
            rc = timeOne(pl, &ms);
            if (rc) {
                delete pl;
                break;
            }
            char line[160];
            std::snprintf(line, sizeof line, "core=%d chunk=%lld%s grid=%s tasks=%d: %.4f ms\n",
                          pl->core, (long long)pl->chunk,
                          pl->overlap ? " overlap" : "",
                          g == 0 ? "all" : g == 1 ? "7/8" : g == 2 ? "3/4" : g == 3 ? "5/8" : "1/2",
                          pl->ntasks, ms);
            rep += line;
            if (!*best || ms < best_ms) {
                delete *best;
                *best = pl;
                best_ms = ms;
            } else {
                delete pl;
            }
        }
    }
    P.tune = saved;
    ce = cudaMemcpyAsync(P.d_states, snap, sbytes, cudaMemcpyDeviceToDevice, S(s));
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(S(s));
    if (!rc && ce != cudaSuccess) rc = cudaErr(ce, "autotune restore");
    cudaFree(snap);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        delete *best;
        *best = nullptr;
        return rc;
    }
    if (*best) {
        const mtgp_gpu_plan *b = *best;
        const char *kern =
            T::kBits == 64 ? (b->core == 2 ? "k_batch64x2 (two words per thread)"
                              : b->split ? "k_batch64 (one word per thread, in-CTA jumps)"
                                         : "k_batch64 (one word per thread)")
            : b->core == 4 ? (b->split ? "k_batch32xk<4> (four words per thread, in-CTA jumps)"
                                       : "k_batch32xk<4> (four words per thread)")
            : b->core == 2 ? (b->split ? "k_batch32xk<2> (two words per thread, in-CTA jumps)"
                                       : "k_batch32xk<2> (two words per thread)")
                           : (b->split ? "k_batch32 (one word per thread, in-CTA jumps)"
                                       : "k_batch32 (one word per thread)");
        char grid[32], pre[64] = "", line[256];
        if (b->grid > 0) std::snprintf(grid, sizeof grid, "%d CTAs", b->grid);
        else std::snprintf(grid, sizeof grid, "all resident");
        if (b->npre)
            // k_jump_part5 is the 48-register form for 32-bit MEXP 11213
            std::snprintf(pre, sizeof pre, " %s %s (%d windows jumped ahead)",
                          b->overlap ? "beside" : "after",
                          T::kBits == 32 && P.sh.mexp == 11213 ? "k_jump_part5" : "k_jump_part",
                          b->npre);
        std::snprintf(line, sizeof line, "chosen: %s%s, chunk=%lld, grid=%s, tasks=%d: %.4f ms\n",
                      kern, pre, (long long)b->chunk, grid, b->ntasks, best_ms);
        rep += line;
    }
    if (report && cap > 0) {
        std::snprintf(report, (size_t)cap, "%s", rep.c_str());
    }
    return MTGP_OK;
}

}  // namespace

extern "C" {

// ---- pools ----------------------------------------------------------------
#define POOL_API(B, W)                                                                           \
    int mtgp##B##_gpu_pool_create(mtgp##B##_gpu_pool_t **out, const mtgp##B##_params_fast_t *p, \
                                  int np, const int *pidx, const W *seeds, int count) {          \
        if (!seeds) return setErr(MTGP_ERR_INVALID, "null seeds");                              \
        int rc = newObj(out);                                                                    \
        if (!rc) rc = (*out)->pool.init(p, np, pidx, count);                                     \
        if (!rc) rc = (*out)->pool.seedAll(seeds);                                               \
        if (rc && out && *out) {                                                                 \
            delete *out;                                                                         \
            *out = nullptr;                                                                      \
        }                                                                                        \
        return rc;                                                                               \
    }                                                                                            \
    int mtgp##B##_gpu_pool_create_by_array(mtgp##B##_gpu_pool_t **out,                           \
                                           const mtgp##B##_params_fast_t *p, int np,             \
                                           const int *pidx, const W *keys,                       \
                                           const uint64_t *key_offsets, int count) {             \
        if (count <= 0 || !key_offsets || (key_offsets[count] > 0 && !keys))                    \
            return setErr(MTGP_ERR_INVALID, "bad key arrays");                                  \
        int rc = newObj(out);                                                                    \
        if (!rc) rc = (*out)->pool.init(p, np, pidx, count);                                     \
        if (!rc) rc = (*out)->pool.seedKeys(keys, key_offsets);                                  \
        if (rc && out && *out) {                                                                 \
            delete *out;                                                                         \
            *out = nullptr;                                                                      \
        }                                                                                        \
        return rc;                                                                               \
    }                                                                                            \
    int mtgp##B##_gpu_pool_create_by_str(mtgp##B##_gpu_pool_t **out,                             \
                                         const mtgp##B##_params_fast_t *p, int np,               \
                                         const int *pidx, const char *const *strs, int count) {  \
        if (count <= 0 || !strs) return setErr(MTGP_ERR_INVALID, "bad key strings");           \
        std::vector<W> keys;                                                                     \
        std::vector<uint64_t> off((size_t)count + 1, 0);                                         \
        for (int i = 0; i < count; i++) {                                                        \
            if (!strs[i]) return setErr(MTGP_ERR_INVALID, "null key string %d", i);            \
            for (const char *c = strs[i]; *c; c++) keys.push_back(T##B::strKey(*c));             \
            off[(size_t)i + 1] = keys.size();                                                    \
        }                                                                                        \
        return mtgp##B##_gpu_pool_create_by_array(out, p, np, pidx, keys.data(), off.data(),    \
                                                  count);                                        \
    }                                                                                            \
    int mtgp##B##_gpu_pool_create_substreams(mtgp##B##_gpu_pool_t **out,                         \
                                             const mtgp##B##_params_fast_t *p, W seed,           \
                                             int count, const uint32_t *table, int rows,         \
                                             int nwords, void *s) {                              \
        int rc = newObj(out);                                                                    \
        if (!rc) rc = (*out)->pool.init(p, 1, nullptr, count);                                   \
        if (!rc) {                                                                               \
            std::vector<W> seeds((size_t)count, seed);                                           \
            rc = (*out)->pool.seedAll(seeds.data());                                             \
        }                                                                                        \
        if (!rc) rc = (*out)->pool.substreams(table, rows, nwords, s);                           \
        if (rc && out && *out) {                                                                 \
            delete *out;                                                                         \
            *out = nullptr;                                                                      \
        }                                                                                        \
        return rc;                                                                               \
    }                                                                                            \
    void mtgp##B##_gpu_pool_free(mtgp##B##_gpu_pool_t *p) {                                      \
        if (!p) return;                                                                          \
        cudaDeviceSynchronize();                                                                 \
        delete p;                                                                                \
    }                                                                                            \
    int mtgp##B##_gpu_pool_size(const mtgp##B##_gpu_pool_t *p) { return p ? p->pool.count : 0; } \
    int mtgp##B##_gpu_pool_fill(mtgp##B##_gpu_pool_t *p, int kind, void *out, size_t n,          \
                                void *s) {                                                       \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        return p->pool.fillAll(kind, out, n, s);                                                 \
    }                                                                                            \
    int mtgp##B##_gpu_pool_fill_stream(mtgp##B##_gpu_pool_t *p, int i, int kind, void *out,      \
                                       size_t n, void *s) {                                      \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        if (kind < 0 || kind > 4) return setErr(MTGP_ERR_INVALID, "unknown kind %d", kind);     \
        return p->pool.fillOne(i, kind, out, n, s);                                              \
    }                                                                                            \
    int mtgp##B##_gpu_pool_plan(mtgp##B##_gpu_pool_t *p, const mtgp_work_item_t *items,          \
                                int nitems, mtgp_gpu_plan_t **plan) {                            \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        if (!plan) return setErr(MTGP_ERR_INVALID, "null plan pointer");                        \
        *plan = nullptr;                                                                         \
        return makePlan(p->pool, items, nitems, plan);                                           \
    }                                                                                            \
    int mtgp##B##_gpu_pool_replan(mtgp##B##_gpu_pool_t *p, const mtgp_work_item_t *items,        \
                                  int nitems, mtgp_gpu_plan_t *plan) {                           \
        if (!p || !plan) return setErr(MTGP_ERR_INVALID, "null pool or plan");                  \
        mtgp_gpu_plan_t *pl = plan;                                                              \
        return makePlan(p->pool, items, nitems, &pl);                                            \
    }                                                                                            \
    int mtgp##B##_gpu_pool_submit(mtgp##B##_gpu_pool_t *p, const mtgp_work_item_t *items,        \
                                  int nitems, void *out, void *s) {                              \
        mtgp_gpu_plan_t *pl = nullptr;                                                           \
        int rc = mtgp##B##_gpu_pool_plan(p, items, nitems, &pl);                                 \
        if (rc) return rc;                                                                       \
        rc = planLaunch(pl, out, s);                                                             \
        cudaError_t e = cudaStreamSynchronize(S(s));                                             \
        delete pl;                                                                               \
        if (!rc && e != cudaSuccess) rc = cudaErr(e, "batched launch");                          \
        return rc;                                                                               \
    }                                                                                            \
    int mtgp##B##_gpu_pool_jump_polys(mtgp##B##_gpu_pool_t *p, int param_set,                   \
                                      const uint64_t *steps, int n, uint32_t *dev_out, void *s) { \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        return p->pool.jumpPolysApi(param_set, steps, n, dev_out, s);                           \
    }                                                                                            \
    int mtgp##B##_gpu_pool_jump_array(mtgp##B##_gpu_pool_t *p, int i, const uint32_t *poly,      \
                                      int nw, void *s) {                                         \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        return p->pool.jumpArray(i, poly, nw, s);                                                \
    }                                                                                            \
    int mtgp##B##_gpu_pool_get_windows_host(mtgp##B##_gpu_pool_t *p, W *w, size_t n) {           \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        return p->pool.getWindows(w, n);                                                         \
    }                                                                                            \
    int mtgp##B##_gpu_pool_set_windows_host(mtgp##B##_gpu_pool_t *p, const W *w, size_t n) {     \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        return p->pool.setWindows(w, n);                                                         \
    }                                                                                            \
    int mtgp##B##_gpu_pool_export(mtgp##B##_gpu_pool_t *p, int i, mtgp##B##_fast_t *dst) {       \
        if (!p) return setErr(MTGP_ERR_INVALID, "null pool");                                   \
        return p->pool.exportTo(i, dst);                                                         \
    }

POOL_API(32, uint32_t)
POOL_API(64, uint64_t)

int mtgp32_gpu_pool_autotune(mtgp32_gpu_pool_t *p, const mtgp_work_item_t *items, int nitems,
                             void *dev_out, void *stream, int reps, mtgp_gpu_plan_t **plan,
                             char *report, int report_cap) {
    if (!p) return setErr(MTGP_ERR_INVALID, "null pool");
    return autotune(p->pool, items, nitems, dev_out, stream, reps, plan, report, report_cap);
}

int mtgp64_gpu_pool_autotune(mtgp64_gpu_pool_t *p, const mtgp_work_item_t *items, int nitems,
                             void *dev_out, void *stream, int reps, mtgp_gpu_plan_t **plan,
                             char *report, int report_cap) {
    if (!p) return setErr(MTGP_ERR_INVALID, "null pool");
    return autotune(p->pool, items, nitems, dev_out, stream, reps, plan, report, report_cap);
}

int mtgp32_gpu_pool_set_tuning(mtgp32_gpu_pool_t *p, const char *key, int64_t value) {
    if (!p) return setErr(MTGP_ERR_INVALID, "null pool");
    return applyTuning(p->pool.tune, key, value);
}
int mtgp64_gpu_pool_set_tuning(mtgp64_gpu_pool_t *p, const char *key, int64_t value) {
    if (!p) return setErr(MTGP_ERR_INVALID, "null pool");
    return applyTuning(p->pool.tune, key, value);
}
}  // extern "C"
