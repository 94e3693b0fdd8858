// host_internal.h -- the host side shared by the C-ABI translation units
// (host.cpp: errors, allocations, tuning defaults; plan.cpp: batched plans;
// single.cpp: single generators; pool_api.cpp: pools and the autotuner).
// Not part of the ABI: the word-size traits, the device-resident stream
// pool, the handle structs and the plan functions the units share.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <atomic>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "batch.h"
#include "gf2.h"
#include "internal.h"
#include "plan_core.h"
#include "pow_sched.h"


namespace mtgp {
namespace host {

// Store a printf-formatted message as the calling thread's
// mtgp_gpu_last_error(); returns code.
int setErr(int code, const char *fmt, ...);

inline int cudaErr(cudaError_t e, const char *what) {
    // an allocation that failed is the reference's -1 (mtgp32-fast.c:47-51)
    return setErr(e == cudaErrorMemoryAllocation ? MTGP_ERR_ALLOC : MTGP_ERR_CUDA, "%s: %s", what,
                  cudaGetErrorString(e));
}

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cudaErr(e_, what); \
    } while (0)

inline cudaStream_t S(void *s) { return static_cast<cudaStream_t>(s); }

// Tuning knobs (mtgp_gpu_set_tuning).  split_chunk: 0 = automatic, < 0 =
// never split long requests, > 0 = split into chunks of this many values.
// batch_grid: 0 = one CTA per resident slot, > 0 = that many CTAs.
// A skip at least this long is done by a GF(2) jump inside the batched
// kernel (about the work of 2^17 generated values) instead of generation.
constexpr uint64_t kJumpMinSkip = 1 << 17;
// Longest skip generated step by step (on exponents without the in-kernel
// jump): about ten seconds of one CTA.
constexpr uint64_t kMaxGenSkip = uint64_t(1) << 34;

// single_chunk: chunk length of split single-generator fills (0 =
// automatic).  jump_parts: CTAs per jump made ahead of a batched launch
// (split single fills, and batched tasks that start with one jump): 0 =
// four, at most one per tap chunk of the jump kernel; -1 = such jumps run
// inside the batched kernel instead.
// core: the 32-bit generation core (2 = two words per thread, 4 = four, 1
// = one); poly_window: bits per comb window of the GPU's polynomial
// products (0 = automatic, 2, 4).  Every pool and single generator carries
// its own copy, taken from the process defaults when it is created, so
// tuning one handle (or changing the defaults) never changes another's plans.
struct Tuning {
    int64_t split_chunk = 0;
    int64_t batch_grid = 0;
    int64_t single_chunk = 0;
    int64_t jump_parts = 0;
    int core = 2;
    int poly_window = 0;
    // jump_overlap: 1 = tasks that start from windows jumped ahead of the
    // launch run in a second persistent launch on a side stream right after
    // the jump parts, while the first launch runs every other task (off by
    // default and not among the autotuner's candidates: those tasks are the
    // longest, and starting them after the jumps lengthens the launch)
    int jump_overlap = 0;
};
inline std::mutex g_tune_mu;
inline Tuning g_tune_default;  // mtgp_gpu_set_tuning: defaults for new handles

inline Tuning tuningDefaults() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune_default;
}

// One tuning key applied to t (the keys of mtgp_gpu_set_tuning).
inline int applyTuning(Tuning &t, const char *key, int64_t value) {
    if (!key) return setErr(MTGP_ERR_INVALID, "null key");
    if (!std::strcmp(key, "split_chunk")) {
        t.split_chunk = value;
    } else if (!std::strcmp(key, "core")) {
        if (value != 1 && value != 2 && value != 4)
            return setErr(MTGP_ERR_INVALID, "core must be 1, 2 or 4");
        t.core = (int)value;
    } else if (!std::strcmp(key, "poly_window")) {
        if (value != 0 && value != 2 && value != 4)
            return setErr(MTGP_ERR_INVALID, "poly_window must be 0, 2 or 4");
        t.poly_window = (int)value;
    } else if (!std::strcmp(key, "batch_grid")) {
        if (value < 0) return setErr(MTGP_ERR_INVALID, "batch_grid must be >= 0");
        t.batch_grid = value;
    } else if (!std::strcmp(key, "single_chunk")) {
        if (value < 0) return setErr(MTGP_ERR_INVALID, "single_chunk must be >= 0");
        t.single_chunk = value;
    } else if (!std::strcmp(key, "jump_parts")) {
        if (value < -1) return setErr(MTGP_ERR_INVALID, "jump_parts must be >= -1");
        t.jump_parts = value;
    } else if (!std::strcmp(key, "jump_overlap")) {
        if (value != 0 && value != 1) return setErr(MTGP_ERR_INVALID, "jump_overlap must be 0 or 1");
        t.jump_overlap = (int)value;
    } else {
        return setErr(MTGP_ERR_INVALID, "unknown tuning key '%s'", key);
    }
    return MTGP_OK;
}

// Jumps made ahead of a batched launch run as four CTAs each: every part
// regenerates the sequence up to its taps, so one CTA per tap chunk (11 for
// MEXP 11213) costs more than it saves (measured on split single fills).
constexpr int kJumpParts = 4;

// CTAs per jump made ahead of a batched launch, for a jump of tchunks tap
// chunks (tuning knob jump_parts).
inline int jumpParts(const Tuning &t, int tchunks) {
    const int64_t p = t.jump_parts > 0 ? t.jump_parts : kJumpParts;
    return (int)std::min<int64_t>(p, tchunks);
}

// ------------------------------------------------------------------------
// Traits of the two word sizes.
// ------------------------------------------------------------------------
struct T32 {
    using W = uint32_t;
    using HP = mtgp32_params_fast_t;
    using DP = DevParams32;
    using Fast = mtgp32_fast_t;
    static constexpr int kBits = 32;
    static bool shape(int mexp, Shape *s) { return shape32(mexp, s); }
    static cudaError_t gen(int mexp, int kind, const DP *p, const int *pi, W *st, int ng,
                           void *out, uint64_t n, uint64_t os, cudaStream_t s, int core) {
        return launchGen32(mexp, kind, p, pi, st, ng, out, n, os, s, core);
    }
    static cudaError_t jump(int mexp, const DP *p, W *st, const JumpDesc *d, int nd, int nw,
                            cudaStream_t s) {
        return launchJump32(mexp, p, st, d, nd, nw, s);
    }
    static cudaError_t batch(const BatchLaunch &b, const DP *p, W *st, cudaStream_t s) {
        return launchBatch32(b, p, st, s);
    }
    static cudaError_t unstage(int mexp, W *st, const void *stage, const int32_t *streams, int n,
                               cudaStream_t s) {
        return launchUnstage32(mexp, st, stage, streams, n, s);
    }
    static cudaError_t parts(int mexp, const DP *p, const W *st, const uint32_t *polys, int nw,
                             W *dst, int stride, const JumpPart *d, int nd, cudaStream_t s) {
        return launchJumpParts32(mexp, p, st, polys, nw, dst, stride, d, nd, s);
    }
    static int jumpChunks(int mexp, int nw) { return jumpChunks32(mexp, nw); }
    static cudaError_t windows(const W *gen, W *win, int n, int stride, int nwin, cudaStream_t s) {
        return launchChunkWindows32(gen, win, n, stride, nwin, s);
    }
    static int resident(int mexp, bool split, int core) {
        return batchResident32(mexp, split, core);
    }
    static bool splits(int mexp) { return batchSplits32(mexp); }
    static cudaError_t seed(const DP *p, const int *pi, const W *seeds, W *st, int n, int size,
                            int stride) {
        return launchSeed32(p, pi, seeds, st, n, size, stride, nullptr);
    }
    static cudaError_t bm(const W *seqs, int n2, int n, int nw, uint32_t *C, int *L) {
        return launchBM32(seqs, n2, n, nw, C, L, nullptr);
    }
    static cudaError_t keyed(const DP *p, const int *pi, const W *keys, const uint64_t *koff,
                             W *st, int n, int size, int stride) {
        return launchKeyed32(p, pi, keys, koff, st, n, size, stride, nullptr);
    }
    // a string byte as the reference adds it to the state: a signed char
    // (its behaviour on x86-64), whatever the host's char signedness
    static W strKey(char c) { return (W)(int)(signed char)c; }
};

struct T64 {
    using W = uint64_t;
    using HP = mtgp64_params_fast_t;
    using DP = DevParams64;
    using Fast = mtgp64_fast_t;
    static constexpr int kBits = 64;
    static bool shape(int mexp, Shape *s) { return shape64(mexp, s); }
    static cudaError_t gen(int mexp, int kind, const DP *p, const int *pi, W *st, int ng,
                           void *out, uint64_t n, uint64_t os, cudaStream_t s, int core) {
        return launchGen64(mexp, kind, p, pi, st, ng, out, n, os, s, core);
    }
    static cudaError_t jump(int mexp, const DP *p, W *st, const JumpDesc *d, int nd, int nw,
                            cudaStream_t s) {
        return launchJump64(mexp, p, st, d, nd, nw, s);
    }
    static cudaError_t batch(const BatchLaunch &b, const DP *p, W *st, cudaStream_t s) {
        return launchBatch64(b, p, st, s);
    }
    static cudaError_t unstage(int mexp, W *st, const void *stage, const int32_t *streams, int n,
                               cudaStream_t s) {
        return launchUnstage64(mexp, st, stage, streams, n, s);
    }
    static cudaError_t parts(int mexp, const DP *p, const W *st, const uint32_t *polys, int nw,
                             W *dst, int stride, const JumpPart *d, int nd, cudaStream_t s) {
        return launchJumpParts64(mexp, p, st, polys, nw, dst, stride, d, nd, s);
    }
    static int jumpChunks(int mexp, int nw) { return jumpChunks64(mexp, nw); }
    static cudaError_t windows(const W *gen, W *win, int n, int stride, int nwin, cudaStream_t s) {
        return launchChunkWindows64(gen, win, n, stride, nwin, s);
    }
    static int resident(int mexp, bool split, int core) {
        return batchResident64(mexp, split, core);
    }
    static bool splits(int mexp) { return batchSplits64(mexp); }
    static cudaError_t seed(const DP *p, const int *pi, const W *seeds, W *st, int n, int size,
                            int stride) {
        return launchSeed64(p, pi, seeds, st, n, size, stride, nullptr);
    }
    static cudaError_t bm(const W *seqs, int n2, int n, int nw, uint32_t *C, int *L) {
        return launchBM64(seqs, n2, n, nw, C, L, nullptr);
    }
    static cudaError_t keyed(const DP *p, const int *pi, const W *keys, const uint64_t *koff,
                             W *st, int n, int size, int stride) {
        return launchKeyed64(p, pi, keys, koff, st, n, size, stride, nullptr);
    }
    static W strKey(char c) { return (W)(int64_t)(int)(signed char)c; }
};

template <class T>
int checkParams(const typename T::HP &p, Shape *sh) {
    if (!T::shape(p.mexp, sh))
        return setErr(MTGP_ERR_UNSUPPORTED, "mtgp%d: Mersenne exponent %d not supported", T::kBits,
                      p.mexp);
    if (p.pos < 1 || p.pos > sh->n - sh->tn)
        return setErr(MTGP_ERR_UNSUPPORTED,
                      "mtgp%d: pos %d outside [1, %d] (needs size - pos >= %d lanes)", T::kBits,
                      p.pos, sh->n - sh->tn, sh->tn);
    if (p.sh1 < 0 || p.sh1 >= 32 || p.sh2 < 0 || p.sh2 >= 32)
        return setErr(MTGP_ERR_INVALID, "mtgp%d: shift out of range", T::kBits);
    return MTGP_OK;
}

// ------------------------------------------------------------------------
// Pool: `count` device-resident streams of one Mersenne exponent.
// ------------------------------------------------------------------------
template <class T>
struct Pool {
    using W = typename T::W;
    Shape sh{};
    int count = 0, nparams = 0, stride = 0, size = 0;
    std::vector<typename T::HP> hparams;
    std::vector<int> hpidx;
    typename T::DP *d_params = nullptr;
    int *d_pidx = nullptr;
    W *d_states = nullptr;
    uint32_t *d_poly = nullptr;
    size_t poly_cap = 0;
    JumpDesc *d_desc = nullptr;
    size_t desc_cap = 0;
    std::vector<gf2::Poly> chi;   // characteristic polynomial per parameter set
    std::vector<int> chideg;
    // Jump arithmetic per parameter set, made on first use: chi's modulus
    // tables and X^(2^i) mod chi for i < 64.
    std::vector<std::unique_ptr<gf2::Modulus>> mod;
    std::vector<std::vector<gf2::Poly>> pow2;
    // X^steps mod chi, keyed by (parameter set, steps); bounded
    std::map<std::pair<int, uint64_t>, gf2::Poly> jcache;
    // Plans of one pool may be made on several threads at once (a server
    // plans each slot's batch on its own thread): the polynomial caches and
    // tables above are read and filled under cache_mu; everything else a
    // plan needs is the plan's own or thread-local.
    std::recursive_mutex cache_mu;
    Tuning tune = tuningDefaults();  // this pool's tuning knobs

    ~Pool() {
        if (cache_stream) cudaStreamSynchronize(cache_stream);
        if (afill.done) cudaEventDestroy(afill.done);
        if (afill.h) cudaFreeHost(afill.h);
        for (uint32_t *b : afill.old) cudaFreeHost(b);
        if (afill.h_ops) cudaFreeHost(afill.h_ops);
        for (unsigned char *b : afill.old_h) cudaFreeHost(b);
        cudaFree(afill.d);
        for (unsigned char *b : afill.old_d) cudaFree(b);
        for (uint32_t *b : gpow_blocks) cudaFree(b);
        if (cache_stream) cudaStreamDestroy(cache_stream);
        cudaFree(d_params);
        cudaFree(d_pidx);
        cudaFree(d_states);
        cudaFree(d_poly);
        cudaFree(d_desc);
    }

    int init(const typename T::HP *params, int np, const int *pidx, int n) {
        if (!params || np <= 0 || n <= 0) return setErr(MTGP_ERR_INVALID, "empty pool");
        int rc = checkParams<T>(params[0], &sh);
        if (rc) return rc;
        for (int k = 1; k < np; k++) {
            Shape s2;
            rc = checkParams<T>(params[k], &s2);
            if (rc) return rc;
            if (s2.mexp != sh.mexp)
                return setErr(MTGP_ERR_INVALID, "pool parameter sets mix exponents %d and %d",
                              sh.mexp, s2.mexp);
        }
        count = n;
        nparams = np;
        size = sh.n;
        stride = stateStride(sh.n);
        hparams.assign(params, params + np);
        hpidx.resize(n);
        for (int i = 0; i < n; i++) {
            int k = pidx ? pidx[i] : (np == n ? i : 0);
            if (k < 0 || k >= np) return setErr(MTGP_ERR_INVALID, "param_idx[%d] = %d out of range", i, k);
            hpidx[i] = k;
        }
        std::vector<typename T::DP> dp(np);
        for (int k = 0; k < np; k++) toDev(params[k], &dp[k]);
        CK(devMalloc(&d_params, sizeof(typename T::DP) * np), "devMalloc(params)");
        CK(devMalloc(&d_pidx, sizeof(int) * n), "devMalloc(pidx)");
        CK(devMalloc(&d_states, sizeof(W) * (size_t)stride * n), "devMalloc(states)");
        CK(cudaMemcpy(d_params, dp.data(), sizeof(typename T::DP) * np, cudaMemcpyHostToDevice),
           "upload params");
        CK(cudaMemcpy(d_pidx, hpidx.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "upload pidx");
        CK(cudaMemset(d_states, 0, sizeof(W) * (size_t)stride * n), "clear states");
        chi.assign(np, gf2::Poly());
        chideg.assign(np, -1);
        powWidth();  // set now: plans read it on several threads
        return MTGP_OK;
    }

    int setWindows(const W *win, size_t nwords) {
        if (!win || nwords < (size_t)count * size)
            return setErr(MTGP_ERR_INVALID, "window buffer too small");
        CK(cudaDeviceSynchronize(), "synchronize");
        CK(cudaMemcpy2D(d_states, sizeof(W) * stride, win, sizeof(W) * size, sizeof(W) * size,
                        count, cudaMemcpyHostToDevice),
           "upload windows");
        return MTGP_OK;
    }

    int getWindows(W *win, size_t nwords) {
        if (!win || nwords < (size_t)count * size)
            return setErr(MTGP_ERR_INVALID, "window buffer too small");
        CK(cudaDeviceSynchronize(), "synchronize");
        CK(cudaMemcpy2D(win, sizeof(W) * size, d_states, sizeof(W) * stride, sizeof(W) * size,
                        count, cudaMemcpyDeviceToHost),
           "download windows");
        return MTGP_OK;
    }

    // Integer seeds, seeded on the device (mtgp32-fast.c:119-137).
    int seedAll(const W *seeds) {
        W *d_seeds = nullptr;
        CK(devMalloc(&d_seeds, sizeof(W) * count), "devMalloc(seeds)");
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess)
            e = cudaMemcpy(d_seeds, seeds, sizeof(W) * count, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = T::seed(d_params, d_pidx, d_seeds, d_states, count, size, stride);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        cudaFree(d_seeds);
        if (e != cudaSuccess) return cudaErr(e, "device seeding");
        return MTGP_OK;
    }

    // Key-schedule seeding of every stream on the device: stream i from the
    // key words keys[koff[i] .. koff[i+1]) (host arrays, koff: count + 1).
    int seedKeys(const W *keys, const uint64_t *koff) {
        const uint64_t nk = koff[count];
        for (int i = 0; i < count; i++)
            if (koff[i + 1] < koff[i] || koff[i + 1] - koff[i] > (uint64_t)INT32_MAX - 2)
                return setErr(MTGP_ERR_INVALID, "bad key offsets at stream %d", i);
        W *d_keys = nullptr;
        uint64_t *d_off = nullptr;
        cudaError_t e = devMalloc(&d_keys, sizeof(W) * (nk ? nk : 1));
        if (e == cudaSuccess) e = devMalloc(&d_off, sizeof(uint64_t) * (count + 1));
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e == cudaSuccess && nk)
            e = cudaMemcpy(d_keys, keys, sizeof(W) * nk, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(d_off, koff, sizeof(uint64_t) * (count + 1), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = T::keyed(d_params, d_pidx, d_keys, d_off, d_states, count, size, stride);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        cudaFree(d_keys);
        cudaFree(d_off);
        if (e != cudaSuccess) return cudaErr(e, "device key schedule");
        return MTGP_OK;
    }

    static int checkKind(int kind) {
        if (kind < 0 || kind > 4) return setErr(MTGP_ERR_INVALID, "unknown output kind %d", kind);
        return MTGP_OK;
    }

    int checkOut(const void *out, size_t n) {
        if (n == 0) return MTGP_OK;
        if (!out) return setErr(MTGP_ERR_INVALID, "null output pointer");
        if (reinterpret_cast<uintptr_t>(out) % sizeof(W))
            return setErr(MTGP_ERR_INVALID, "output pointer not %zu-byte aligned", sizeof(W));
        return MTGP_OK;
    }

    int fillAll(int kind, void *out, size_t n, void *s) {
        int rc = checkKind(kind);
        if (!rc) rc = checkOut(out, n);
        if (rc) return rc;
        CK(T::gen(sh.mexp, kind, d_params, d_pidx, d_states, count, out, n, n, S(s), tune.core),
           "generate");
        return MTGP_OK;
    }

    int fillOne(int i, int kind, void *out, size_t n, void *s) {
        if (i < 0 || i >= count) return setErr(MTGP_ERR_INVALID, "stream %d out of range", i);
        int rc = kind == -1 ? MTGP_OK : checkKind(kind);
        if (!rc && kind >= 0) rc = checkOut(out, n);
        if (rc) return rc;
        CK(T::gen(sh.mexp, kind, d_params, d_pidx + i, d_states + (size_t)i * stride, 1, out, n, n,
                  S(s), tune.core),
           "generate");
        return MTGP_OK;
    }

    int maxPolyWords() const { return 2 * (sh.mexp / 32 + 1); }

    int ensureScratch(size_t words, size_t descs) {
        if (words > poly_cap) {
            cudaFree(d_poly);
            d_poly = nullptr;
            CK(devMalloc(&d_poly, sizeof(uint32_t) * words), "devMalloc(poly)");
            poly_cap = words;
        }
        if (descs > desc_cap) {
            cudaFree(d_desc);
            d_desc = nullptr;
            CK(devMalloc(&d_desc, sizeof(JumpDesc) * descs), "devMalloc(jump descriptors)");
            desc_cap = descs;
        }
        return MTGP_OK;
    }

    // Jump stream i by one polynomial (uint32-array form).
    int jumpArray(int i, const uint32_t *poly, int nwords, void *s) {
        if (i < 0 || i >= count) return setErr(MTGP_ERR_INVALID, "stream %d out of range", i);
        if (!poly || nwords <= 0) return setErr(MTGP_ERR_BAD_JUMP, "empty jump polynomial");
        while (nwords > 1 && poly[nwords - 1] == 0) nwords--;
        if (nwords > maxPolyWords())
            return setErr(MTGP_ERR_BAD_JUMP, "jump polynomial of %d words exceeds %d", nwords,
                          maxPolyWords());
        int rc = ensureScratch((size_t)nwords, 1);
        if (rc) return rc;
        // The scratch buffers are reused: order this call after earlier ones.
        CK(cudaStreamSynchronize(S(s)), "synchronize");
        CK(cudaMemcpy(d_poly, poly, sizeof(uint32_t) * nwords, cudaMemcpyHostToDevice),
           "upload polynomial");
        JumpDesc d{};
        d.poly[0] = d_poly;
        d.nchain = 1;
        d.pidx = hpidx[i];
        d.src = d.dst = (uint64_t)i * stride;
        CK(cudaMemcpy(d_desc, &d, sizeof d, cudaMemcpyHostToDevice), "upload descriptor");
        CK(T::jump(sh.mexp, d_params, d_states, d_desc, 1, nwords, S(s)), "jump");
        return MTGP_OK;
    }

    int fastJump(int i, const char *hex, void *s) {
        if (!hex) return setErr(MTGP_ERR_BAD_JUMP, "null jump string");
        gf2::Poly p;
        int ncoef = 0;
        if (!gf2::fromHex(hex, &p, &ncoef))
            return setErr(MTGP_ERR_BAD_JUMP, "jump string has a non-hex character");
        int nw = std::max(1, (ncoef + 31) / 32);
        std::vector<uint32_t> w = gf2::toWords32(p, nw);
        return jumpArray(i, w.data(), nw, s);
    }

    // Characteristic polynomials of the parameter sets `ks` not yet known, all
    // at once: the LSBs of 2 * mexp outputs of each set from seed 1 (the kind
    // of sequence mtgp32-calc-poly.cpp:36-45 feeds NTL's MinPolySeq),
    // generated on the GPU by a throw-away pool, then Berlekamp-Massey on the
    // GPU, one warp per set (bm_kernels.cu).  chi is the reciprocal of the
    // connection polynomial.
    int characteristics(const std::vector<int> &ks) {
        std::vector<int> miss;
        for (int k : ks)
            if (chideg[k] < 0 && std::find(miss.begin(), miss.end(), k) == miss.end())
                miss.push_back(k);
        if (miss.empty()) return MTGP_OK;
        const int n = (int)miss.size();
        std::vector<typename T::HP> hp;
        for (int k : miss) hp.push_back(hparams[k]);
        Pool<T> tmp;
        int rc = tmp.init(hp.data(), n, nullptr, n);
        if (rc) return rc;
        std::vector<W> ones((size_t)n, (W)1);
        rc = tmp.seedAll(ones.data());
        if (rc) return rc;
        const size_t n2 = 2 * (size_t)sh.mexp;
        const int nw = sh.mexp / 32 + 2;
        W *d_out = nullptr;
        uint32_t *d_C = nullptr;
        int *d_L = nullptr;
        cudaError_t e = devMalloc(&d_out, sizeof(W) * n2 * n);
        if (e == cudaSuccess) e = devMalloc(&d_C, sizeof(uint32_t) * (size_t)nw * n);
        if (e == cudaSuccess) e = devMalloc(&d_L, sizeof(int) * n);
        if (e == cudaSuccess) rc = tmp.fillAll(0, d_out, n2, nullptr);
        if (e == cudaSuccess && !rc) e = T::bm(d_out, (int)n2, n, nw, d_C, d_L);
        std::vector<uint32_t> C((size_t)nw * n);
        std::vector<int> L((size_t)n);
        if (e == cudaSuccess && !rc)
            e = cudaMemcpy(C.data(), d_C, sizeof(uint32_t) * C.size(), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && !rc)
            e = cudaMemcpy(L.data(), d_L, sizeof(int) * n, cudaMemcpyDeviceToHost);
        cudaFree(d_out);
        cudaFree(d_C);
        cudaFree(d_L);
        if (rc) return rc;
        if (e != cudaSuccess) return cudaErr(e, "characteristic polynomials on the GPU");
        for (int j = 0; j < n; j++) {
            const int d = L[(size_t)j];
            if (d != sh.mexp)
                return setErr(MTGP_ERR_UNSUPPORTED,
                              "characteristic polynomial has degree %d, not %d", d, sh.mexp);
            const uint32_t *c = C.data() + (size_t)j * nw;
            gf2::Poly out((size_t)d / 64 + 1, 0);
            for (int i = 0; i <= d; i++) {  // chi_i = C_{d-i}
                const int q = d - i;
                if ((c[q >> 5] >> (q & 31)) & 1u) out[(size_t)i >> 6] |= 1ULL << (i & 63);
            }
            chi[miss[(size_t)j]] = out;
            chideg[miss[(size_t)j]] = d;
        }
        return MTGP_OK;
    }
    int characteristic(int k) { return characteristics({k}); }

    int polyWords() const { return sh.mexp / 32 + 1; }

    // chi_k's reduction tables (2.9 MB for MEXP 11213).  At most kMaxModuli
    // are kept per pool; the least recently used is dropped (and rebuilt in
    // about 2 ms if needed again), so pools with many parameter sets stay
    // small.  A pointer handed out stays valid until the next call for
    // another parameter set.
    static constexpr int kMaxModuli = 16;
    std::vector<uint64_t> mod_used;
    uint64_t mod_clock = 0;
    int modulus(int k, const gf2::Modulus **out) {
        int rc = characteristic(k);
        if (rc) return rc;
        if (mod.size() < hparams.size()) {
            mod.resize(hparams.size());
            mod_used.resize(hparams.size(), 0);
        }
        if (!mod[k]) {
            int live = 0, lru = -1;
            for (size_t j = 0; j < mod.size(); j++)
                if (mod[j]) {
                    live++;
                    if (lru < 0 || mod_used[j] < mod_used[(size_t)lru]) lru = (int)j;
                }
            if (live >= kMaxModuli) mod[(size_t)lru].reset();
            mod[k].reset(new (std::nothrow) gf2::Modulus(chi[k], chideg[k]));
        }
        if (!mod[k]) return setErr(MTGP_ERR_ALLOC, "jump tables");
        mod_used[k] = ++mod_clock;
        *out = mod[k].get();
        return MTGP_OK;
    }

    // X^(2^i) mod chi_k for i < 64 (host copies of the device table's slots).
    int ensurePow2(int k) {
        if (pow2.size() < hparams.size()) pow2.resize(hparams.size());
        if (!pow2[k].empty()) return MTGP_OK;
        return prepare({k});
    }

    // Device tables for computing X^e mod chi_k on the GPU (pow_sched.h):
    // chi | mu = floor(X^(2D) / chi) | slot 256m + k = X^(k 2^(8m)) mod chi,
    // polyWords() words each (2.9 MB for MEXP 11213).  prepare() makes them
    // for many parameter sets at once, all on the GPU:
    //   - chi by Berlekamp-Massey (characteristics), mu by the power-series
    //     inverse of chi's reciprocal (bm_kernels.cu), one warp per set;
    //   - X^(2^i): monomials while 2^i < D, then one squaring per level
    //     (products of k_powops, every set in the same launch);
    //   - the other slots by tableSchedule (seven launches for all sets).
    // The host keeps chi and copies of X^(2^i) (pow2) for its own paths.
    std::map<int, uint32_t *> gpow;
    std::vector<uint32_t *> gpow_blocks;  // allocations holding the tables
    cudaStream_t cache_stream = nullptr;   // startFill's products
    int prepare(const std::vector<int> &ks) {
        std::vector<int> miss;
        for (int k : ks)
            if (!gpow.count(k) && std::find(miss.begin(), miss.end(), k) == miss.end())
                miss.push_back(k);
        if (miss.empty()) return MTGP_OK;
        const int W = polyWords();
        if (!powOpsFits(W)) return setErr(MTGP_ERR_UNSUPPORTED, "polynomials too long for the GPU");
        int rc = characteristics(miss);
        if (rc) return rc;
        const int n = (int)miss.size(), D = sh.mexp;
        const size_t TW = (size_t)(2 + kPowSlots) * W;  // words of one set's table
        std::vector<uint32_t> h_chi((size_t)n * W);
        for (int j = 0; j < n; j++) {
            const std::vector<uint32_t> w = gf2::toWords32(chi[miss[(size_t)j]], W);
            std::copy(w.begin(), w.end(), h_chi.begin() + (std::ptrdiff_t)((size_t)j * W));
        }
        // products: squarings X^(2^i) = (X^(2^(i-1)))^2 from the first 2^i >= D,
        // one level each, then the byte-window table levels
        int i0 = 0;
        while (i0 < 64 && (uint64_t(1) << i0) < (uint64_t)D) i0++;
        PowSchedule sq;
        for (int i = i0 > 0 ? i0 : 1; i < 64; i++) {
            std::vector<PowStep> lev;
            for (int j = 0; j < n; j++) {
                PowStep st{};
                st.job = j;
                st.nsrc = 2;
                st.src[0] = st.src[1] = powSlot((i - 1) / 8, 1 << ((i - 1) % 8));
                st.dst = powSlot(i / 8, 1 << (i % 8));
                lev.push_back(st);
            }
            sq.levels.push_back(std::move(lev));
        }
        PowSchedule one, tabs;
        tableSchedule(one);
        tabs.levels.resize(one.levels.size());
        for (size_t l = 0; l < one.levels.size(); l++)
            for (int j = 0; j < n; j++)
                for (PowStep st : one.levels[l]) {
                    st.job = j;
                    tabs.levels[l].push_back(st);
                }
        // host <-> device copies are plain 1D copies of contiguous staging
        // (chi in, X^(2^i) out); the scatter and gather run on the device
        uint32_t *blk = nullptr, *stage = nullptr;
        PowOp *d_ops = nullptr;
        cudaStream_t st = nullptr;
        const size_t nstage = (size_t)n * 64 * W;  // >= n * W (chi)
        cudaError_t e = devMalloc(&blk, sizeof(uint32_t) * TW * n);
        if (e == cudaSuccess) e = devMalloc(&stage, sizeof(uint32_t) * nstage);
        if (e == cudaSuccess)
            e = devMalloc(&d_ops, sizeof(PowOp) * (size_t)(sq.steps() + tabs.steps()));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMemsetAsync(blk, 0, sizeof(uint32_t) * TW * n, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(stage, h_chi.data(), sizeof(uint32_t) * h_chi.size(),
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)  // chi into word 0 of each table
            e = cudaMemcpy2DAsync(blk, sizeof(uint32_t) * TW, stage, sizeof(uint32_t) * W,
                                  sizeof(uint32_t) * W, n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = launchBarrett(blk, D, n, W, TW, blk + W, st);
        if (e == cudaSuccess) e = launchMonomials(blk, TW, W, n, i0, st);  // X^(2^i), 2^i < D
        std::vector<PowOp> ops, more;
        auto tab = [&](int j) { return (const uint32_t *)(blk + (size_t)j * TW); };
        powOpsTo(sq, tab, blk + 2 * (size_t)W, TW, D, ops);
        powOpsTo(tabs, tab, blk + 2 * (size_t)W, TW, D, more);
        ops.insert(ops.end(), more.begin(), more.end());
        if (e == cudaSuccess && !ops.empty())
            e = cudaMemcpyAsync(d_ops, ops.data(), sizeof(PowOp) * ops.size(),
                                cudaMemcpyHostToDevice, st);
        size_t first = 0;
        for (const PowSchedule *sc : {&sq, &tabs})
            for (size_t l = 0; e == cudaSuccess && l < sc->levels.size(); l++) {
                const int m = (int)sc->levels[l].size();
                e = launchPowOps(d_ops + first, m, nullptr, W, st, tune.poly_window);
                first += (size_t)m;
            }
        // host copies of X^(2^i)
        std::vector<uint32_t> h_p2(nstage);
        if (e == cudaSuccess) e = launchGatherPow2(blk, TW, W, n, stage, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess)
            e = cudaMemcpy(h_p2.data(), stage, sizeof(uint32_t) * nstage, cudaMemcpyDeviceToHost);
        if (st) cudaStreamDestroy(st);
        cudaFree(d_ops);
        cudaFree(stage);
        if (e != cudaSuccess) {
            cudaFree(blk);
            return cudaErr(e, "jump tables on the GPU");
        }
        gpow_blocks.push_back(blk);
        if (pow2.size() < hparams.size()) pow2.resize(hparams.size());
        for (int j = 0; j < n; j++) {
            const int k = miss[(size_t)j];
            gpow[k] = blk + (size_t)j * TW;
            std::vector<gf2::Poly> &P2 = pow2[k];
            P2.assign(64, gf2::Poly());
            for (int i = 0; i < 64; i++)
                P2[(size_t)i] = gf2::fromWords32(h_p2.data() + ((size_t)j * 64 + i) * W, W);
        }
        return MTGP_OK;
    }
    int gpuPowTables(int k, const uint32_t **out) {
        int rc = prepare({k});
        if (rc) return rc;
        *out = gpow.at(k);
        return MTGP_OK;
    }

    // Device form of a schedule whose output codes are table slots of each
    // job's table (dst = dst_base + job * job_stride + slot * W).
    template <class Tab>
    void powOpsTo(const PowSchedule &sch, Tab tab, uint32_t *dst_base, size_t job_stride, int D,
                  std::vector<PowOp> &ops) const {
        const size_t W = (size_t)polyWords();
        ops.clear();
        for (const auto &lev : sch.levels)
            for (const PowStep &st : lev) {
                PowOp o{};
                o.tab = tab(st.job);
                o.dst = dst_base + (size_t)st.job * job_stride + (size_t)st.dst * W;
                o.D = D;
                o.nsrc = st.nsrc;
                for (int q = 0; q < kPowMaxSrc; q++) o.src[q] = st.src[q];
                ops.push_back(o);
            }
    }

    // Device form of a schedule, level by level: table slots of tab(job),
    // scratch slots of `scratch`, outputs at dst_base + index * W.
    template <class Tab>
    void powOps(const PowSchedule &sch, Tab tab, uint32_t *dst_base, uint32_t *scratch, int D,
                std::vector<PowOp> &ops) const {
        const size_t W = (size_t)polyWords();
        ops.clear();
        for (const auto &lev : sch.levels)
            for (const PowStep &st : lev) {
                PowOp o{};
                o.tab = tab(st.job);
                o.dst = st.dst >= 0 ? dst_base + (size_t)st.dst * W
                                    : scratch + (size_t)(-1 - st.dst) * W;
                o.D = D;
                o.nsrc = st.nsrc;
                for (int q = 0; q < kPowMaxSrc; q++) o.src[q] = st.src[q];
                ops.push_back(o);
            }
    }

    // CTAs of the product kernel that run at once (one per SM).
    int pow_width = 0;
    int powWidth() {
        if (!pow_width) {
            int dev = 0, sms = 152;
            if (cudaGetDevice(&dev) == cudaSuccess)
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            pow_width = sms > 0 ? sms : 152;
        }
        return pow_width;
    }

    // X^steps mod chi for (parameter set, steps) pairs not yet in the host
    // cache, computed on the GPU together (the tables of all their sets made
    // first, in one prepare) and put in the cache once they are back: a
    // later plan's cache step (harvestFill) takes them.  No caller waits for
    // the GPU here: products queued behind batches in flight would stall
    // every plan of the pool.  One fill is in flight at a time; a plan that
    // misses a polynomial makes it itself, on the GPU at its launch.
    // harvestFill with cache_mu held; startFill takes it for its bookkeeping
    // only, not while it queues the GPU work.
    struct AsyncFill {
        std::vector<std::pair<int, uint64_t>> keys;
        uint32_t *h = nullptr;  // pinned: the products come back here
        size_t cap = 0;         // words of h
        std::vector<uint32_t *> old;  // smaller buffers, freed with the pool
        // device buffer (products | ops | scratch) and pinned ops, kept and
        // grown (an allocation on the way could wait for the GPU)
        unsigned char *d = nullptr, *h_ops = nullptr;
        size_t dcap = 0, h_ops_cap = 0;
        std::vector<unsigned char *> old_d, old_h;
        cudaEvent_t done = nullptr;
        bool busy = false;       // a fill is being queued or is in flight
        bool submitted = false;  // ... and `done` is recorded after it
    } afill;

    void harvestFill() {
        if (!afill.busy || !afill.submitted || cudaEventQuery(afill.done) != cudaSuccess) return;
        const int W = polyWords();
        if (jcache.size() + afill.keys.size() > 16384) jcache.clear();
        for (size_t j = 0; j < afill.keys.size(); j++)
            jcache[afill.keys[j]] = gf2::fromWords32(afill.h + j * (size_t)W, W);
        afill.keys.clear();
        afill.busy = false;
        afill.submitted = false;
    }

    int startFill(const std::vector<std::pair<int, uint64_t>> &want) {
        std::vector<std::pair<int, uint64_t>> need;
        std::vector<const uint32_t *> tabs;
        {
            std::lock_guard<std::recursive_mutex> lk(cache_mu);
            harvestFill();
            if (afill.busy) return MTGP_OK;
            for (const auto &q : want)
                if (!jcache.count(q) && std::find(need.begin(), need.end(), q) == need.end())
                    need.push_back(q);
            if (need.empty()) return MTGP_OK;
            std::vector<int> sets;
            for (const auto &q : need) sets.push_back(q.first);
            int rc = prepare(sets);
            if (rc) return rc;
            if (!cache_stream)
                CK(cudaStreamCreateWithFlags(&cache_stream, cudaStreamNonBlocking),
                   "cudaStreamCreate(cache)");
            if (!afill.done)
                CK(cudaEventCreateWithFlags(&afill.done, cudaEventDisableTiming),
                   "cudaEventCreate(cache)");
            for (const auto &q : need) tabs.push_back(gpow.at(q.first));
            afill.busy = true;  // this thread owns afill until it is submitted
        }
        int rc = queueFill(need, tabs);
        std::lock_guard<std::recursive_mutex> lk(cache_mu);
        if (rc) {
            afill.busy = false;
            return rc;
        }
        afill.keys = std::move(need);
        afill.submitted = true;
        return MTGP_OK;
    }

    // The GPU work of a fill (startFill owns afill meanwhile).
    int queueFill(const std::vector<std::pair<int, uint64_t>> &need,
                  const std::vector<const uint32_t *> &tabs) {
        const int W = polyWords(), n = (int)need.size();
        if ((size_t)n * W > afill.cap) {  // no fill in flight reads the old buffer
            if (afill.h) afill.old.push_back(afill.h);
            afill.h = nullptr;
            afill.cap = 0;
            const size_t cap = std::max<size_t>(2 * (size_t)n * W, (size_t)64 * W);
            CK(hostAlloc(&afill.h, sizeof(uint32_t) * cap), "cudaMallocHost(cache products)");
            afill.cap = cap;
        }
        std::vector<uint64_t> steps((size_t)n);
        for (int j = 0; j < n; j++) steps[(size_t)j] = need[(size_t)j].second;
        PowSchedule sch;
        powSchedule(steps.data(), n, powWidth(), sch);
        // on the pool's own stream, in buffers that only grow (freeing one
        // would wait for every batch in flight; no fill is in flight here)
        const size_t out_bytes = sizeof(uint32_t) * (size_t)n * W;
        const size_t ops_bytes = (sizeof(PowOp) * (size_t)sch.steps() + 255) & ~size_t(255);
        const size_t bytes = ((out_bytes + 255) & ~size_t(255)) + ops_bytes +
                             sizeof(uint32_t) * (size_t)sch.nscratch * W;
        if (bytes > afill.dcap) {
            if (afill.d) afill.old_d.push_back(afill.d);
            afill.d = nullptr;
            afill.dcap = 0;
            CK(devMalloc(&afill.d, 2 * bytes), "cudaMalloc(cache products)");
            afill.dcap = 2 * bytes;
        }
        if (ops_bytes > afill.h_ops_cap) {
            if (afill.h_ops) afill.old_h.push_back(afill.h_ops);
            afill.h_ops = nullptr;
            afill.h_ops_cap = 0;
            CK(hostAlloc(&afill.h_ops, 2 * ops_bytes), "cudaMallocHost(cache ops)");
            afill.h_ops_cap = 2 * ops_bytes;
        }
        unsigned char *d = afill.d;
        uint32_t *d_out = reinterpret_cast<uint32_t *>(d);
        PowOp *d_ops = reinterpret_cast<PowOp *>(d + ((out_bytes + 255) & ~size_t(255)));
        uint32_t *d_scratch = reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(d_ops) +
                                                           ops_bytes);
        std::vector<PowOp> &ops = afill_ops;
        ops.clear();
        powOps(sch, [&tabs](int j) { return tabs[(size_t)j]; }, d_out, d_scratch, sh.mexp, ops);
        std::memcpy(afill.h_ops, ops.data(), sizeof(PowOp) * ops.size());
        cudaError_t e = cudaMemcpyAsync(d_ops, afill.h_ops, sizeof(PowOp) * ops.size(),
                                        cudaMemcpyHostToDevice, cache_stream);
        size_t first = 0;
        for (size_t l = 0; e == cudaSuccess && l < sch.levels.size(); l++) {
            const int m = (int)sch.levels[l].size();
            e = launchPowOps(d_ops + first, m, d_scratch, W, cache_stream, tune.poly_window);
            first += (size_t)m;
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(afill.h, d_out, out_bytes, cudaMemcpyDeviceToHost, cache_stream);
        if (e == cudaSuccess) e = cudaEventRecord(afill.done, cache_stream);
        if (e != cudaSuccess) return cudaErr(e, "jump polynomials on the GPU");
        return MTGP_OK;
    }
    std::vector<PowOp> afill_ops;

    // Public form: host exponents, device output (mtgp*_gpu_pool_jump_polys).
    int jumpPolysApi(int k, const uint64_t *steps, int n, uint32_t *out, void *s) {
        if (k < 0 || k >= nparams) return setErr(MTGP_ERR_INVALID, "parameter set %d out of range", k);
        if (n < 0 || (n > 0 && (!steps || !out))) return setErr(MTGP_ERR_INVALID, "bad arguments");
        if (n == 0) return MTGP_OK;
        return gpuPolys(k, steps, n, out, s);
    }

    // X^steps[j] mod chi_k for j < n into out + j * polyWords() (device),
    // ordered on stream s; the tables are made first if needed.
    int gpuPolys(int k, const uint64_t *steps, int n, uint32_t *out, void *s) {
        const uint32_t *t = nullptr;
        int rc = gpuPowTables(k, &t);  // before any stream work
        if (rc) return rc;
        const int W = polyWords();
        PowSchedule sch;
        powSchedule(steps, n, powWidth(), sch);
        unsigned char *d = nullptr;
        const size_t ops_bytes = (sizeof(PowOp) * (size_t)sch.steps() + 255) & ~size_t(255);
        const size_t bytes = ops_bytes + sizeof(uint32_t) * (size_t)sch.nscratch * W;
        CK(devMallocAsync(reinterpret_cast<void **>(&d), bytes, S(s)), "devMallocAsync(products)");
        uint32_t *scratch = reinterpret_cast<uint32_t *>(d + ops_bytes);
        std::vector<PowOp> ops;
        powOps(sch, [t](int) { return t; }, out, scratch, chideg[k], ops);
        cudaError_t e = cudaMemcpyAsync(d, ops.data(), sizeof(PowOp) * ops.size(),
                                        cudaMemcpyHostToDevice, S(s));
        size_t first = 0;
        for (size_t l = 0; e == cudaSuccess && l < sch.levels.size(); l++) {
            const int m = (int)sch.levels[l].size();
            e = launchPowOps(reinterpret_cast<const PowOp *>(d) + first, m, scratch, W, S(s),
                             tune.poly_window);
            first += (size_t)m;
        }
        cudaError_t f = cudaFreeAsync(d, S(s));
        if (e != cudaSuccess) return cudaErr(e, "jump polynomials");
        if (f != cudaSuccess) return cudaErr(f, "cudaFreeAsync");
        return MTGP_OK;
    }

    // Jump stream i ahead by `steps` values: X^steps mod chi made on the GPU
    // (a fraction of a millisecond for any 64-bit distance), then applied.
    int jumpGpu(int i, uint64_t steps, void *s) {
        if (i < 0 || i >= count) return setErr(MTGP_ERR_INVALID, "stream %d out of range", i);
        const int W = polyWords();
        int rc = ensureScratch((size_t)W, 1);
        if (rc) return rc;
        // The scratch buffers are reused: order this call after earlier ones.
        CK(cudaStreamSynchronize(S(s)), "synchronize");
        rc = gpuPolys(hpidx[i], &steps, 1, d_poly, s);
        if (rc) return rc;
        JumpDesc d{};
        d.poly[0] = d_poly;
        d.nchain = 1;
        d.pidx = hpidx[i];
        d.src = d.dst = (uint64_t)i * stride;
        CK(cudaMemcpy(d_desc, &d, sizeof d, cudaMemcpyHostToDevice), "upload descriptor");
        CK(T::jump(sh.mexp, d_params, d_states, d_desc, 1, W, S(s)), "jump");
        return MTGP_OK;
    }

    // X^steps mod chi_k (host, cached): X^(steps - low) * X^low with low the
    // lowest set bit, X^(2^i) cached per parameter set, so that a sequence of
    // multiples of one chunk length costs one product each.
    int jumpPoly(int k, uint64_t steps, const gf2::Poly **out) {
        auto hit = jcache.find({k, steps});
        if (hit != jcache.end()) {
            *out = &hit->second;
            return MTGP_OK;
        }
        int rc = ensurePow2(k);
        if (rc) return rc;
        const std::vector<gf2::Poly> &P2 = pow2[k];
        gf2::Poly r;
        if (steps == 0) {
            r.assign(P2[0].size(), 0);
            r[0] = 1;
        } else {
            const uint64_t low = steps & (~steps + 1);
            int b = 0;
            while ((uint64_t(1) << b) != low) b++;
            if (steps == low) {
                r = P2[b];
            } else {  // a product on the host (the planner fills the cache on the GPU)
                const gf2::Poly *rest = nullptr;
                rc = jumpPoly(k, steps - low, &rest);
                if (rc) return rc;
                const gf2::Poly rest_copy = *rest;  // the cache may be cleared below
                const gf2::Modulus *M = nullptr;
                rc = modulus(k, &M);
                if (rc) return rc;
                r = M->mulmod(rest_copy, pow2[k][b]);
            }
        }
        if (jcache.size() >= 16384) jcache.clear();
        *out = &jcache.emplace(std::make_pair(k, steps), std::move(r)).first->second;
        return MTGP_OK;
    }

    int jumpSteps(int i, uint64_t lo, uint64_t hi, void *s) {
        if (i < 0 || i >= count) return setErr(MTGP_ERR_INVALID, "stream %d out of range", i);
        if (lo == 0 && hi == 0) return MTGP_OK;
        if (hi == 0 && powOpsFits(polyWords())) return jumpGpu(i, lo, s);
        int k = hpidx[i];
        int rc = characteristic(k);
        if (rc) return rc;
        std::vector<uint32_t> e = {(uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi,
                                   (uint32_t)(hi >> 32)};
        const gf2::Modulus *M = nullptr;
        rc = modulus(k, &M);
        if (rc) return rc;
        gf2::Poly p = M->powx(e);
        int nw = chideg[k] / 32 + 1;
        std::vector<uint32_t> w = gf2::toWords32(p, nw);
        return jumpArray(i, w.data(), nw, s);
    }

    // Substream j = stream 0's window jumped by j * step (table rows as in
    // cuda-sample/mtgp32-jump-kernel.cuh:383-401: bit b of j applies row
    // b/2 once for even b, twice for odd b).
    int substreams(const uint32_t *table, int rows, int nwords, void *s) {
        if (!table || rows <= 0 || nwords <= 0 || nwords > maxPolyWords())
            return setErr(MTGP_ERR_BAD_JUMP, "bad jump table");
        if (rows < 16 && (uint64_t)count > (1ULL << (2 * rows)))
            return setErr(MTGP_ERR_INVALID, "%d substreams need more than %d table rows", count,
                          rows);
        int rc = ensureScratch((size_t)rows * nwords, (size_t)count);
        if (rc) return rc;
        CK(cudaStreamSynchronize(S(s)), "synchronize");
        CK(cudaMemcpy(d_poly, table, sizeof(uint32_t) * rows * nwords, cudaMemcpyHostToDevice),
           "upload jump table");
        // Doubling: level k makes windows [2^k, 2^(k+1)) from windows
        // [0, 2^k), each by one jump of X^(2^k * step) = table row k/2,
        // applied twice for odd k (the table holds the steps 4^r * step).
        // Window j then went through the rows of the reference's table walk
        // (cuda-sample/mtgp32-jump-kernel.cuh:383-401: bit b of j applies
        // row b/2 once or twice, lowest bit first) in the same order, so the
        // windows are bit-identical to it, with one jump per substream
        // instead of up to 2 * rows; the levels run one launch each.
        std::vector<JumpDesc> descs;
        descs.reserve(count);
        std::vector<int> level_end;
        for (int k = 0; k < 31 && (1 << k) < count; k++) {
            if (k / 2 >= rows)
                return setErr(MTGP_ERR_INVALID, "%d substreams need more than %d table rows",
                              count, rows);
            const uint32_t *row = d_poly + (size_t)(k / 2) * nwords;
            for (int j = 0; j < (1 << k) && j + (1 << k) < count; j++) {
                JumpDesc d{};
                d.poly[d.nchain++] = row;
                if (k & 1) d.poly[d.nchain++] = row;
                d.pidx = hpidx[j];
                d.src = (uint64_t)j * stride;
                d.dst = (uint64_t)(j + (1 << k)) * stride;
                descs.push_back(d);
            }
            level_end.push_back((int)descs.size());
        }
        if (descs.empty()) return MTGP_OK;
        CK(cudaMemcpy(d_desc, descs.data(), sizeof(JumpDesc) * descs.size(),
                      cudaMemcpyHostToDevice),
           "upload descriptors");
        int first = 0;
        for (int end : level_end) {
            CK(T::jump(sh.mexp, d_params, d_states, d_desc + first, end - first, nwords, S(s)),
               "jump");
            first = end;
        }
        return MTGP_OK;
    }

    int exportTo(int i, typename T::Fast *dst) {
        if (i < 0 || i >= count) return setErr(MTGP_ERR_INVALID, "stream %d out of range", i);
        if (!dst || !dst->status) return setErr(MTGP_ERR_INVALID, "destination has no status");
        const typename T::HP &p = hparams[hpidx[i]];
        int ls = 1;
        while (ls <= size) ls <<= 1;
        if (dst->status->size != size || dst->status->large_size != ls)
            return setErr(MTGP_ERR_INVALID,
                          "destination status has size %d / large_size %d, expected %d / %d",
                          dst->status->size, dst->status->large_size, size, ls);
        CK(cudaDeviceSynchronize(), "synchronize");
        CK(cudaMemcpy(dst->status->array, d_states + (size_t)i * stride, sizeof(W) * size,
                      cudaMemcpyDeviceToHost),
           "download window");
        dst->params = p;
        dst->status->idx = size - 1;
        dst->status->large_mask = ls - 1;
        return MTGP_OK;
    }
};


// Whether a pool's plans may start tasks from jumped windows: with the
// in-kernel jump (MEXP 11213 and 23209), or else with jumps made ahead of
// the launch by jump parts (every exponent, unless jump_parts = -1).
template <class T>
bool planJumps(const Pool<T> &P) {
    return T::splits(P.sh.mexp) || P.tune.jump_parts >= 0;
}

// Shortest skip (and chunk) worth a jump.  A jump's correlation costs about
// N * mexp word XORs (N window words; twice for 64-bit words), as much as
// generating ~2^17 values at MEXP 11213; the exponents without the
// in-kernel jump scale that by their cost, to a power of two (2^21 for
// 44497, 2^24 for 64-bit 110503).
template <class T>
uint64_t jumpMinSkip(const Pool<T> &P) {
    if (T::splits(P.sh.mexp)) return kJumpMinSkip;
    const double rel = (double)P.sh.n * P.sh.mexp * (T::kBits / 32) / (351.0 * 11213.0);
    uint64_t m = kJumpMinSkip;
    while ((double)m < (double)kJumpMinSkip * rel) m <<= 1;
    return m;
}


}  // namespace host
}  // namespace mtgp

using namespace mtgp;
using namespace mtgp::host;

// ---- the handle structs of the C ABI --------------------------------------
// Large fills of a single generator run split over many CTAs (see
// fillSingle).  Two slots of buffers are used in turn, so a fill never
// rewrites buffers that the GPU may still be reading for the previous one.
struct SingleFill {
    // chunk-start jump polynomials X^(c * poly_chunk) mod chi, c = 1..npolys
    // (device, polyWords words each), kept while the chunk length stays
    uint32_t *d_polys = nullptr;
    size_t cap_polys = 0;
    int64_t poly_chunk = 0;
    int npolys = 0;
    struct Slot {
        void *d_win = nullptr;  // chunk-start windows
        size_t cap_win = 0;
        unsigned char *h_desc = nullptr, *d_desc = nullptr;  // tasks | items | parts
        size_t cap_desc = 0;
        unsigned *d_counter = nullptr;
        // what the uploaded descriptors describe
        size_t n = 0;
        int kind = -9, parts = 0;
        int64_t chunk = 0;
        const void *win = nullptr, *polys = nullptr;
        mtgp_gpu_plan *plan = nullptr;  // jump_parts = -1: a split plan
    } slot[2];
    cudaEvent_t done[2] = {nullptr, nullptr};
    int next = 0;
};
struct mtgp32_gpu {
    Pool<T32> pool;
    SingleFill fill;
};
struct mtgp64_gpu {
    Pool<T64> pool;
    SingleFill fill;
};
struct mtgp32_gpu_pool { Pool<T32> pool; };
struct mtgp64_gpu_pool { Pool<T64> pool; };

struct mtgp_gpu_plan {
    int bits = 32;
    void *pool = nullptr;  // Pool<T32> or Pool<T64>
    int ntasks = 0;
    int mode = -2;         // shared output kind of all items, or -2 (mixed)
    uint64_t out_bytes = 0;
    int grid = 0;
    bool split = false;    // some tasks start with an in-kernel jump
    int core = 4;          // 32-bit generation core of unsplit plans
    int64_t chunk = 0;     // chunk length used when splitting
    int nstage = 0;
    // Descriptors (tasks | items | jump polynomials | staged streams), built
    // in pinned host memory and uploaded by one asynchronous copy on the
    // stream of the next launch; both buffers are kept and only grown, so a
    // server can refill plans without allocating (cudaFree and cudaFreeHost
    // would wait for every batch in flight).
    unsigned char *h_blob = nullptr, *d_blob = nullptr;
    size_t cap_h = 0, cap_d = 0, blob_bytes = 0;
    bool dirty = false;
    const BatchTask *d_tasks = nullptr;
    const BatchItem *d_items = nullptr;
    const uint32_t *d_polys = nullptr;
    const int32_t *d_stage_streams = nullptr;
    unsigned *d_counter = nullptr;
    // jump polynomials computed on the GPU before each launch, after the
    // host-computed ones: the product levels of pow_sched.h (steps per
    // level, one launch each), their scratch polynomials kept and grown
    std::vector<int> pow_levels;
    bool pow_ready = true;  // false from an upload until the products have run
    const PowOp *d_powops = nullptr;
    uint32_t *d_pscratch = nullptr;
    size_t cap_pscratch = 0;
    void *d_stage = nullptr;  // final windows of streams with several tasks
    size_t cap_stage = 0;
    // jumps made ahead of the launch (BatchTask::pre): npre windows, each the
    // sum of its jump's parts (nparts descriptors in the blob), made before
    // every launch into slots that are zero (zeroed at allocation, and by the
    // batched kernel as each task reads its slot)
    // A task that jumps twice takes its window from a second launch of parts
    // (nparts_b, after the first nparts), which jump the run starts made by
    // the first launch in nmid middle slots (after the npre tasks' slots;
    // cleared after each launch) by the chunk offsets.
    int npre = 0, nparts = 0, nmid = 0, nparts_b = 0;
    const JumpPart *d_parts = nullptr;
    void *d_prewin = nullptr;
    size_t cap_prewin = 0;
    bool prewin_fresh = false;  // allocated, not yet zeroed
    // jump_overlap: tasks [nmain, ntasks) start from pre-jumped windows and
    // run in a second persistent launch on `side`, after the jump parts
    // there, beside the launch of tasks [0, nmain) on the caller's stream
    // (fork and join by events, so a graph capture takes both)
    bool overlap = false;
    int nmain = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;

    cudaGraphExec_t exec = nullptr;
    void *graph_out = nullptr;
    // buffers replaced by larger ones, freed with the plan
    std::vector<void *> retired_dev, retired_host;
    ~mtgp_gpu_plan() {
        for (void *b : retired_dev) cudaFree(b);
        for (void *b : retired_host) cudaFreeHost(b);
        if (exec) cudaGraphExecDestroy(exec);
        if (side) cudaStreamDestroy(side);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        cudaFree(d_stage);
        cudaFree(d_prewin);
        cudaFree(d_pscratch);
        cudaFree(d_blob);
        cudaFreeHost(h_blob);
        cudaFree(d_counter);
    }
};


namespace mtgp {
namespace host {

// Batched plans (plan.cpp).  makePlan builds (or, given *out, refills) a
// plan for the items; launchPlan runs it on a stream; planLaunch picks the
// word size.
template <class T>
int makePlan(Pool<T> &P, const mtgp_work_item_t *items, int nitems, mtgp_gpu_plan **out,
             int force_core = 0, int64_t force_chunk = 0);
template <class T>
int launchPlan(mtgp_gpu_plan *pl, void *out, void *s);
int planLaunch(mtgp_gpu_plan *pl, void *out, void *s);

template <class Obj>
int newObj(Obj **out) {
    if (!out) return setErr(MTGP_ERR_INVALID, "null output handle pointer");
    *out = new (std::nothrow) Obj();
    if (!*out) return setErr(MTGP_ERR_ALLOC, "host allocation failed");
    return MTGP_OK;
}

}  // namespace host
}  // namespace mtgp
