// host.cpp -- the C ABI of include/mtgp_gpu.h.
//
// Host side of the GB300 MTGP generator: parameter validation, seeding (the
// reference's exact integer arithmetic, done once per stream on the host as
// the reference's CUDA samples do, cuda-sample/mtgp32-cuda.cu:304-330),
// device memory for parameters and state windows, and the launches of the
// generation, jump and batched kernels.  Everything that produces random
// numbers runs on the GPU; there is no CPU generation path.
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

// Allocation wrappers with the test hook MTGP_TEST_FAIL_ALLOC (internal.h).
namespace {
std::atomic<long long> g_alloc_count{0};
long long failAllocAt() {
    static const long long k = [] {
        const char *v = std::getenv("MTGP_TEST_FAIL_ALLOC");
        return v && *v ? std::atoll(v) : -1LL;
    }();
    return k;
}
bool injectFailure() {
    const long long k = failAllocAt();
    return k >= 0 && g_alloc_count.fetch_add(1) == k;
}
}  // namespace

cudaError_t devMallocRaw(void **p, size_t bytes) {
    if (injectFailure()) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}
cudaError_t devMallocAsyncRaw(void **p, size_t bytes, cudaStream_t s) {
    if (injectFailure()) return cudaErrorMemoryAllocation;
    return cudaMallocAsync(p, bytes, s);
}
cudaError_t hostAllocRaw(void **p, size_t bytes) {
    if (injectFailure()) return cudaErrorMemoryAllocation;
    return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

void toDev(const mtgp32_params_fast_t &p, DevParams32 *d) {
    std::memset(d, 0, sizeof *d);
    d->pos = p.pos;
    d->sh1 = p.sh1;
    d->sh2 = p.sh2;
    d->mask = p.mask;
    std::memcpy(d->tbl, p.tbl, sizeof d->tbl);
    std::memcpy(d->tmp, p.tmp_tbl, sizeof d->tmp);
    std::memcpy(d->flt, p.flt_tmp_tbl, sizeof d->flt);
}

void toDev(const mtgp64_params_fast_t &p, DevParams64 *d) {
    std::memset(d, 0, sizeof *d);
    d->pos = p.pos;
    d->sh1 = p.sh1;
    d->sh2 = p.sh2;
    d->mask = p.mask;
    std::memcpy(d->tbl, p.tbl, sizeof d->tbl);
    std::memcpy(d->tmp, p.tmp_tbl, sizeof d->tmp);
    std::memcpy(d->dbl, p.dbl_tmp_tbl, sizeof d->dbl);
}

}  // namespace mtgp

using namespace mtgp;

namespace {

thread_local std::string g_err;

int setErr(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

}  // namespace

int mtgp::recordError(int code, const char *msg) { return setErr(code, "%s", msg); }

namespace {

int cudaErr(cudaError_t e, const char *what) {
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
std::mutex g_tune_mu;
Tuning g_tune_default;  // mtgp_gpu_set_tuning: defaults for new handles

Tuning tuningDefaults() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune_default;
}

// One tuning key applied to t (the keys of mtgp_gpu_set_tuning).
int applyTuning(Tuning &t, const char *key, int64_t value) {
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
int jumpParts(const Tuning &t, int tchunks) {
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
                           void *out, uint64_t n, uint64_t os, cudaStream_t s, int) {
        return launchGen64(mexp, kind, p, pi, st, ng, out, n, os, s);
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
    static int resident(int mexp, bool split, int) { return batchResident64(mexp, split); }
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
    cudaStream_t cache_stream = nullptr;   // fillCache's products
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
    // first, in one prepare) and kept in the cache.
    int fillCache(const std::vector<std::pair<int, uint64_t>> &want) {
        std::vector<std::pair<int, uint64_t>> need;
        for (const auto &q : want)
            if (!jcache.count(q) && std::find(need.begin(), need.end(), q) == need.end())
                need.push_back(q);
        if (need.empty()) return MTGP_OK;
        std::vector<int> sets;
        for (const auto &q : need) sets.push_back(q.first);
        int rc = prepare(sets);
        if (rc) return rc;
        const int W = polyWords(), n = (int)need.size();
        std::vector<uint64_t> steps((size_t)n);
        std::vector<const uint32_t *> tabs((size_t)n);
        for (int j = 0; j < n; j++) {
            steps[(size_t)j] = need[(size_t)j].second;
            tabs[(size_t)j] = gpow.at(need[(size_t)j].first);
        }
        PowSchedule sch;
        powSchedule(steps.data(), n, powWidth(), sch);
        // the pool's own stream and stream-ordered allocations: no
        // device-wide synchronization (a cudaFree would wait for every batch
        // in flight), the host waits only for these products
        if (!cache_stream) CK(cudaStreamCreateWithFlags(&cache_stream, cudaStreamNonBlocking),
                              "cudaStreamCreate(cache)");
        const size_t out_bytes = sizeof(uint32_t) * (size_t)n * W;
        const size_t ops_bytes = (sizeof(PowOp) * (size_t)sch.steps() + 255) & ~size_t(255);
        const size_t bytes = ((out_bytes + 255) & ~size_t(255)) + ops_bytes +
                             sizeof(uint32_t) * (size_t)sch.nscratch * W;
        unsigned char *d = nullptr;
        CK(devMallocAsync(reinterpret_cast<void **>(&d), bytes, cache_stream),
           "devMallocAsync(cache products)");
        uint32_t *d_out = reinterpret_cast<uint32_t *>(d);
        PowOp *d_ops = reinterpret_cast<PowOp *>(d + ((out_bytes + 255) & ~size_t(255)));
        uint32_t *d_scratch = reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(d_ops) +
                                                           ops_bytes);
        std::vector<PowOp> ops;
        powOps(sch, [&tabs](int j) { return tabs[(size_t)j]; }, d_out, d_scratch, sh.mexp, ops);
        cudaError_t e = cudaMemcpyAsync(d_ops, ops.data(), sizeof(PowOp) * ops.size(),
                                        cudaMemcpyHostToDevice, cache_stream);
        size_t first = 0;
        for (size_t l = 0; e == cudaSuccess && l < sch.levels.size(); l++) {
            const int m = (int)sch.levels[l].size();
            e = launchPowOps(d_ops + first, m, d_scratch, W, cache_stream, tune.poly_window);
            first += (size_t)m;
        }
        std::vector<uint32_t> h((size_t)n * W);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h.data(), d_out, out_bytes, cudaMemcpyDeviceToHost, cache_stream);
        cudaError_t f = cudaFreeAsync(d, cache_stream);
        if (e == cudaSuccess) e = f;
        if (e == cudaSuccess) e = cudaStreamSynchronize(cache_stream);
        if (e != cudaSuccess) return cudaErr(e, "jump polynomials on the GPU");
        if (jcache.size() + need.size() > 16384) jcache.clear();
        for (int j = 0; j < n; j++)
            jcache[need[(size_t)j]] = gf2::fromWords32(h.data() + (size_t)j * W, W);
        return MTGP_OK;
    }

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

}  // namespace

// ==========================================================================
// Public structs
// ==========================================================================
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
    int npre = 0, nparts = 0;
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
    ~mtgp_gpu_plan() {
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

namespace {

// A jump polynomial X^steps mod chi_pidx computed on the GPU at launch.
struct GpuJob {
    int pidx;
    uint64_t steps;
    int32_t slot;
    const uint32_t *tab;  // the device tables of parameter set pidx
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

template <class T>
int makePlan(Pool<T> &P, const mtgp_work_item_t *items, int nitems, mtgp_gpu_plan **out,
             int force_core = 0, int64_t force_chunk = 0) {
    using W = typename T::W;
    if (!out) return setErr(MTGP_ERR_INVALID, "null plan pointer");
    if (*out && (*out)->pool != &P) return setErr(MTGP_ERR_INVALID, "plan belongs to another pool");
    PlanOptions o;
    o.nstreams = P.count;
    o.word_bytes = sizeof(W);
    // without the in-kernel jump every jumped start is made ahead of the
    // launch, from one polynomial (a run start and a chunk offset combined)
    const bool kernel_jumps = T::splits(P.sh.mexp);
    o.can_jump = planJumps(P);
    o.jump_min = jumpMinSkip(P);
    o.max_gen_skip = kMaxGenSkip;
    o.chunk_tune = force_chunk ? force_chunk : P.tune.split_chunk;
    // Plans whose generated values mix kinds (a generated skip counts as
    // kind -1) run on the one-word core, whose per-kind loops are out of line
    // at no cost.  The same rule as planCore's mode, decided up front because
    // the chunk length depends on the core's resident CTAs.
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
    const int core = force_core ? force_core : (T::kBits == 32 && kinds == -2) ? 1 : P.tune.core;
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
        std::lock_guard<std::recursive_mutex> lk(P.cache_mu);
        auto hit = poly_at.find({pidx, steps});
        if (hit == poly_at.end()) {
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
    // every parameter set that jumps gets its tables in one batch, and the
    // chunk offsets not yet cached are computed together on the GPU
    {
        std::vector<int> sets;
        std::vector<std::pair<int, uint64_t>> offs;
        for (const PlanTask &pt : R.tasks) {
            if (!pt.run && !pt.off) continue;
            const int k = P.hpidx[pt.stream];
            if (std::find(sets.begin(), sets.end(), k) == sets.end()) sets.push_back(k);
            if (pt.off && __builtin_popcountll(pt.off) >= 2) offs.emplace_back(k, pt.off);
        }
        std::lock_guard<std::recursive_mutex> lk(P.cache_mu);
        rc = P.prepare(sets);
        if (!rc) rc = P.fillCache(offs);
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
        if (pt.run && pt.off && !kernel_jumps) {
            rc = polyIndex(t.pidx, pt.run + pt.off, &t.j0, true);
        } else if (pt.run && pt.off) {
            rc = polyIndex(t.pidx, pt.run, &t.j0, true);
            if (!rc) rc = polyIndex(t.pidx, pt.off, &t.j1, false);
        } else if (pt.run || pt.off) {
            rc = polyIndex(t.pidx, pt.run | pt.off, &t.j0, pt.run != 0);
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
    static thread_local std::vector<JumpPart> jparts;
    jparts.clear();
    int npre = 0;
    if (P.tune.jump_parts >= 0 && npolys > 0) {
        const int tch = T::jumpChunks(P.sh.mexp, (int)pw);
        const int parts = jumpParts(P.tune, tch);
        for (BatchTask &t : tasks) {
            if (t.j0 < 0 || t.j1 >= 0) continue;
            for (int q = 0; q < parts; q++) {
                JumpPart d{};
                d.src = (uint64_t)t.stream * (uint64_t)P.stride;
                d.poly = t.j0;
                d.dst = npre;
                d.pidx = t.pidx;
                d.ch0 = (int16_t)(q * tch / parts);
                d.ch1 = (int16_t)((q + 1) * tch / parts);
                jparts.push_back(d);
            }
            t.pre = ++npre;
            t.j0 = -1;
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
    pl->core = pl->mode == -2 ? 1 : core;
    pl->chunk = cut ? chunk : 0;
    pl->nstage = (int)stage_streams.size();
    pl->npre = npre;
    pl->nparts = (int)jparts.size();
    pl->overlap = nmain < (int)tasks.size();
    pl->nmain = nmain;
    auto align = [](size_t n) { return (n + 255) & ~size_t(255); };
    const size_t off_items = align(sizeof(BatchTask) * tasks.size());
    const size_t off_polys = off_items + align(sizeof(BatchItem) * bitems.size());
    const size_t off_ops = off_polys + align(sizeof(uint32_t) * pw * npolys);
    const size_t off_parts = off_ops + align(sizeof(PowOp) * (size_t)sch.steps());
    const size_t off_ss = off_parts + align(sizeof(JumpPart) * jparts.size());
    const size_t bytes = off_ss + sizeof(int32_t) * stage_streams.size();
    cudaError_t e = cudaSuccess;
    if (!pl->d_counter) e = devMalloc(&pl->d_counter, 2 * sizeof(unsigned));
    if (e == cudaSuccess && pl->overlap && !pl->side) {
        e = cudaStreamCreateWithFlags(&pl->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pl->join, cudaEventDisableTiming);
    }
    if (e == cudaSuccess && bytes > pl->cap_d) {
        cudaFree(pl->d_blob);
        pl->d_blob = nullptr;
        pl->cap_d = 0;
        e = devMalloc(&pl->d_blob, bytes + bytes / 4);
        if (e == cudaSuccess) pl->cap_d = bytes + bytes / 4;
    }
    if (e == cudaSuccess && bytes > pl->cap_h) {
        cudaFreeHost(pl->h_blob);
        pl->h_blob = nullptr;
        pl->cap_h = 0;
        e = hostAlloc(&pl->h_blob, bytes + bytes / 4);
        if (e == cudaSuccess) pl->cap_h = bytes + bytes / 4;
    }
    if (e == cudaSuccess && (size_t)sch.nscratch * pw > pl->cap_pscratch) {
        const size_t need = (size_t)sch.nscratch * pw;
        cudaFree(pl->d_pscratch);
        pl->d_pscratch = nullptr;
        pl->cap_pscratch = 0;
        e = devMalloc(&pl->d_pscratch, sizeof(uint32_t) * (need + need / 4));
        if (e == cudaSuccess) pl->cap_pscratch = need + need / 4;
    }
    if (e == cudaSuccess && pl->nstage) {
        const size_t need = sizeof(W) * (size_t)P.stride * pl->nstage;
        if (need > pl->cap_stage) {
            cudaFree(pl->d_stage);
            pl->d_stage = nullptr;
            pl->cap_stage = 0;
            e = devMalloc(&pl->d_stage, need + need / 4);
            if (e == cudaSuccess) pl->cap_stage = need + need / 4;
        }
    }
    if (e == cudaSuccess && pl->npre) {
        const size_t need = sizeof(W) * (size_t)P.stride * pl->npre;
        if (need > pl->cap_prewin) {
            cudaFree(pl->d_prewin);
            pl->d_prewin = nullptr;
            pl->cap_prewin = 0;
            e = devMalloc(&pl->d_prewin, need + need / 4);
            if (e == cudaSuccess) pl->cap_prewin = need + need / 4;
            pl->prewin_fresh = true;
        }
    }
    if (e != cudaSuccess) {
        if (fresh) {
            delete pl;
        } else {  // a refilled plan that could not grow launches nothing
            pl->ntasks = 0;
            pl->nstage = 0;
            pl->npre = 0;
            pl->nparts = 0;
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

// n successive values of one generator.  A fill of at least kSplitFillMin
// values, on an exponent with GF(2) jumps, is cut into chunks: chunk c starts
// from the generator's window jumped by X^(c * chunk) mod chi.  Those windows
// are made first, every jump's correlation split over several CTAs
// (k_jump_part, a range of the jump kernel's tap chunks each), from
// polynomials kept on the device for the chunk length; then one batched
// launch runs every chunk from its window on the two-word core, with no jump
// inside it, and the window after the last chunk becomes the generator's.
// A 2^20-value fill takes 0.05 ms this way (0.12 ms with one in-kernel jump
// per chunk, 0.41 ms on one CTA), 2^26 values 0.18 ms.  Smaller fills,
// and fills issued while the stream is being captured, run on one CTA.  The
// first split fill of a parameter set also computes its characteristic
// polynomial and jump tables (tens of milliseconds, and a device
// synchronisation), and a new chunk length its chunk polynomials.
constexpr size_t kSplitFillMin = size_t(1) << 20;
constexpr int64_t kMaxFillChunks = 4096;

// Chunk length of a split fill of n values: the power of two nearest to
// 32 sqrt(n) for MEXP 11213 (measured on GB300: 2^15 for 2^20 values, 2^18
// for 2^26; more chunks cost more jumps, longer ones a longer run), scaled
// by mexp / 11213 (a jump's correlation grows with mexp^2, so the best
// length grows with mexp).

int64_t singleChunk(size_t n, int mexp) {
    const double t = 32.0 * (mexp / 11213.0) * std::sqrt((double)n);
    int64_t c = 1;
    while ((double)c * 1.4142135623730951 < t) c <<= 1;
    return c;
}

int waitSlot(SingleFill &F, int i) {
    if (F.done[i])
        CK(cudaEventSynchronize(F.done[i]), "wait for an earlier fill");
    else
        CK(cudaEventCreateWithFlags(&F.done[i], cudaEventDisableTiming), "cudaEventCreate");
    return MTGP_OK;
}

template <class T, class Obj>
int fillSingle(Obj *h, int kind, void *out, size_t n, void *s);

int planLaunch(mtgp_gpu_plan *pl, void *out, void *s) {
    return pl->bits == 32 ? launchPlan<T32>(pl, out, s) : launchPlan<T64>(pl, out, s);
}

// The same fill as a one-item split plan whose chunks start with in-kernel
// jumps, one CTA per jump, on the one-word core (tuning knob jump_parts =
// -1; about two chunks per SM).
template <class T, class Obj>
int fillSplitPlan(Obj *h, int kind, void *out, size_t n, void *s, int sms) {
    Pool<T> &P = h->pool;
    SingleFill &F = h->fill;
    const int i = F.next;
    int rc = waitSlot(F, i);
    if (rc) return rc;
    mtgp_work_item_t it{};
    it.stream = 0;
    it.kind = kind;
    it.count = n;
    int64_t chunk = P.tune.split_chunk;
    if (chunk == 0) {
        chunk = 1 << 17;
        while ((uint64_t)chunk * 2 * (uint64_t)sms < n) chunk <<= 1;
    }
    rc = makePlan(P, &it, 1, &F.slot[i].plan, 1, chunk);
    if (!rc) rc = launchPlan<T>(F.slot[i].plan, out, s);
    if (rc) return rc;
    CK(cudaEventRecord(F.done[i], S(s)), "record fill");
    F.next ^= 1;
    return MTGP_OK;
}

template <class T, class Obj>
int fillSingle(Obj *h, int kind, void *out, size_t n, void *s) {
    using W = typename T::W;
    Pool<T> &P = h->pool;
    if (n < kSplitFillMin || !T::splits(P.sh.mexp)) return P.fillAll(kind, out, n, s);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(S(s), &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return P.fillAll(kind, out, n, s);
    int rc = P.checkKind(kind);
    if (!rc) rc = P.checkOut(out, n);
    if (rc) return rc;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (P.tune.jump_parts < 0) return fillSplitPlan<T>(h, kind, out, n, s, sms);
    int64_t chunk = P.tune.single_chunk > 0 ? P.tune.single_chunk : singleChunk(n, P.sh.mexp);
    if ((n + chunk - 1) / chunk > (uint64_t)kMaxFillChunks)
        chunk = (int64_t)((n + kMaxFillChunks - 1) / kMaxFillChunks);
    const int nch = (int)((n + chunk - 1) / chunk);
    if (nch < 2) return P.fillAll(kind, out, n, s);
    SingleFill &F = h->fill;
    const int i = F.next;
    SingleFill::Slot &L = F.slot[i];
    rc = waitSlot(F, i);
    if (rc) return rc;

    // chunk-start polynomials X^(c * chunk), c = 1 .. nch - 1
    const int pw = P.polyWords();
    if (F.poly_chunk != chunk || F.npolys < nch - 1) {
        for (int q = 0; q < 2; q++)  // earlier fills may still read them
            if (F.done[q]) CK(cudaEventSynchronize(F.done[q]), "wait for an earlier fill");
        const size_t words = (size_t)(nch - 1) * (size_t)pw;
        F.poly_chunk = 0;
        F.npolys = 0;
        if (words > F.cap_polys) {
            cudaFree(F.d_polys);
            F.d_polys = nullptr;
            F.cap_polys = 0;
            CK(devMalloc(&F.d_polys, sizeof(uint32_t) * words), "devMalloc(chunk polynomials)");
            F.cap_polys = words;
        }
        std::vector<uint64_t> steps((size_t)nch - 1);
        for (int c = 1; c < nch; c++) steps[(size_t)c - 1] = (uint64_t)c * (uint64_t)chunk;
        rc = P.gpuPolys(P.hpidx[0], steps.data(), nch - 1, F.d_polys, s);
        if (rc) return rc;
        // later fills may be issued on other streams
        CK(cudaStreamSynchronize(S(s)), "chunk polynomials");
        F.poly_chunk = chunk;
        F.npolys = nch - 1;
    }

    // windows, and descriptors (rebuilt only when the fill's shape changes)
    const size_t stride = (size_t)P.stride;
    const size_t win_bytes = sizeof(W) * stride * (size_t)nch;
    if (win_bytes > L.cap_win) {
        cudaFree(L.d_win);
        L.d_win = nullptr;
        L.cap_win = 0;
        CK(devMalloc(&L.d_win, win_bytes), "devMalloc(chunk windows)");
        L.cap_win = win_bytes;
    }
    if (!L.d_counter) CK(devMalloc(&L.d_counter, sizeof(unsigned)), "devMalloc(counter)");
    W *win = static_cast<W *>(L.d_win);
    const int tchunks = T::jumpChunks(P.sh.mexp, pw);
    const int parts = jumpParts(P.tune, tchunks);
    const int nparts = (nch - 1) * parts;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t off_items = al(sizeof(BatchTask) * (size_t)nch);
    const size_t off_parts = off_items + al(sizeof(BatchItem) * (size_t)nch);
    const size_t bytes = off_parts + sizeof(JumpPart) * (size_t)nparts;
    if (L.n != n || L.kind != kind || L.chunk != chunk || L.parts != parts || L.win != L.d_win ||
        L.polys != F.d_polys) {
        L.n = 0;
        if (bytes > L.cap_desc) {
            cudaFreeHost(L.h_desc);
            cudaFree(L.d_desc);
            L.h_desc = L.d_desc = nullptr;
            L.cap_desc = 0;
            CK(hostAlloc(&L.h_desc, bytes), "cudaMallocHost(fill descriptors)");
            CK(devMalloc(&L.d_desc, bytes), "devMalloc(fill descriptors)");
            L.cap_desc = bytes;
        }
        BatchTask *t = reinterpret_cast<BatchTask *>(L.h_desc);
        BatchItem *it = reinterpret_cast<BatchItem *>(L.h_desc + off_items);
        JumpPart *jp = reinterpret_cast<JumpPart *>(L.h_desc + off_parts);
        for (int c = 0; c < nch; c++) {
            t[c] = BatchTask{};
            t[c].stream = c;
            t[c].first = c;
            t[c].nitems = 1;
            t[c].pidx = P.hpidx[0];
            t[c].j0 = t[c].j1 = -1;
            t[c].wb = c == nch - 1 ? kWbStream : kWbNone;
            it[c] = BatchItem{};
            it[c].out_off = (uint64_t)c * (uint64_t)chunk * sizeof(W);
            it[c].count = c == nch - 1 ? n - (uint64_t)c * (uint64_t)chunk : (uint64_t)chunk;
            it[c].kind = kind;
        }
        for (int c = 1; c < nch; c++)
            for (int q = 0; q < parts; q++) {
                JumpPart &d = jp[(size_t)(c - 1) * parts + q];
                d = JumpPart{};
                d.src = 0;
                d.poly = c - 1;
                d.dst = c;
                d.pidx = P.hpidx[0];
                d.ch0 = (int16_t)(q * tchunks / parts);
                d.ch1 = (int16_t)((q + 1) * tchunks / parts);
            }
        CK(cudaMemcpyAsync(L.d_desc, L.h_desc, bytes, cudaMemcpyHostToDevice, S(s)),
           "upload fill descriptors");
        L.n = n;
        L.kind = kind;
        L.chunk = chunk;
        L.parts = parts;
        L.win = L.d_win;
        L.polys = F.d_polys;
    }

    CK(T::windows(P.d_states, win, P.size, (int)stride, nch, S(s)), "chunk windows");
    CK(T::parts(P.sh.mexp, P.d_params, win, F.d_polys, pw, win, (int)stride,
                reinterpret_cast<const JumpPart *>(L.d_desc + off_parts), nparts, S(s)),
       "chunk-start jumps");
    BatchLaunch b{};
    b.mexp = P.sh.mexp;
    b.mode = kind;
    b.grid = std::min(nch, T::resident(P.sh.mexp, false, 2));
    b.core = 2;
    b.split = false;
    b.nwords = pw;
    b.tasks = reinterpret_cast<const BatchTask *>(L.d_desc);
    b.ntasks = nch;
    b.items = reinterpret_cast<const BatchItem *>(L.d_desc + off_items);
    b.out = out;
    b.counter = L.d_counter;
    CK(T::batch(b, P.d_params, win, S(s)), "chunks");
    CK(cudaMemcpyAsync(P.d_states, win + (size_t)(nch - 1) * stride, sizeof(W) * (size_t)P.size,
                       cudaMemcpyDeviceToDevice, S(s)),
       "window after the last chunk");
    CK(cudaEventRecord(F.done[i], S(s)), "record fill");
    F.next ^= 1;
    return MTGP_OK;
}

// Advance one generator by n steps: generated (and discarded) below
// kSkipJumpMin steps, a GF(2) jump by X^n mod chi above (the polynomial made
// on the GPU; a few launches instead of n steps).
constexpr uint64_t kSkipJumpMin = uint64_t(1) << 22;

template <class T>
int skipSingle(Pool<T> &P, uint64_t n, void *s) {
    if (n < kSkipJumpMin) return P.fillOne(0, -1, nullptr, n, s);
    return P.jumpGpu(0, n, s);
}

template <class Obj>
void freeSingle(Obj *h) {
    cudaDeviceSynchronize();
    SingleFill &F = h->fill;
    for (int i = 0; i < 2; i++) {
        SingleFill::Slot &L = F.slot[i];
        delete L.plan;
        cudaFree(L.d_win);
        cudaFree(L.d_desc);
        cudaFreeHost(L.h_desc);
        cudaFree(L.d_counter);
        if (F.done[i]) cudaEventDestroy(F.done[i]);
    }
    cudaFree(F.d_polys);
    delete h;
}

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
    const int cores[3] = {4, 2, 1};
    const int ncores = T::kBits == 32 ? 3 : 1;
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
                          T::kBits == 64 ? 1 : pl->core, (long long)pl->chunk,
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
            T::kBits == 64 ? (b->split ? "k_batch64 (one word per thread, in-CTA jumps)"
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

template <class Obj>
int newObj(Obj **out) {
    if (!out) return setErr(MTGP_ERR_INVALID, "null output handle pointer");
    *out = new (std::nothrow) Obj();
    if (!*out) return setErr(MTGP_ERR_ALLOC, "host allocation failed");
    return MTGP_OK;
}

// A single generator from an integer seed, seeded on the device.
template <class T, class Obj>
int initSeeded(Obj **out, const typename T::HP *para, typename T::W seed) {
    int rc = newObj(out);
    if (rc) return rc;
    rc = (*out)->pool.init(para, 1, nullptr, 1);
    if (!rc) rc = (*out)->pool.seedAll(&seed);
    if (rc) {
        delete *out;
        *out = nullptr;
    }
    return rc;
}

// A single generator from a key schedule (init_by_array / init_by_str),
// seeded on the device.
template <class T, class Obj>
int initKeyed(Obj **out, const typename T::HP *para, const typename T::W *keys, int len) {
    int rc = newObj(out);
    if (rc) return rc;
    const uint64_t koff[2] = {0, (uint64_t)len};
    rc = (*out)->pool.init(para, 1, nullptr, 1);
    if (!rc) rc = (*out)->pool.seedKeys(keys, koff);
    if (rc) {
        delete *out;
        *out = nullptr;
    }
    return rc;
}

template <class T>
std::vector<typename T::W> strKeys(const char *str) {
    std::vector<typename T::W> k(std::strlen(str));
    for (size_t j = 0; j < k.size(); j++) k[j] = T::strKey(str[j]);
    return k;
}

template <class T, class Obj>
int importSingle(Obj *h, const typename T::Fast *src) {
    using W = typename T::W;
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    if (!src || !src->status) return setErr(MTGP_ERR_INVALID, "source has no status");
    Shape sh;
    int rc = checkParams<T>(src->params, &sh);
    if (rc) return rc;
    if (sh.mexp != h->pool.sh.mexp)
        return setErr(MTGP_ERR_INVALID, "source exponent %d differs from handle's %d", sh.mexp,
                      h->pool.sh.mexp);
    const int size = h->pool.size;
    int ls = src->status->large_size, idx = src->status->idx;
    if (src->status->size != size || ls <= size || (ls & (ls - 1)))
        return setErr(MTGP_ERR_INVALID, "source status has unexpected sizes");
    std::vector<W> win(size);
    for (int k = 0; k < size; k++) win[k] = src->status->array[(idx - size + 1 + k + ls) & (ls - 1)];
    typename T::DP dp;
    toDev(src->params, &dp);
    CK(cudaDeviceSynchronize(), "synchronize");
    CK(cudaMemcpy(h->pool.d_params, &dp, sizeof dp, cudaMemcpyHostToDevice), "upload params");
    h->pool.hparams[0] = src->params;
    h->pool.chideg[0] = -1;
    return h->pool.setWindows(win.data(), win.size());
}

}  // namespace

// ==========================================================================
// C ABI
// ==========================================================================
extern "C" {

const char *mtgp_gpu_last_error(void) { return g_err.c_str(); }
const char *mtgp_gpu_version(void) { return "mtgp-gb300 0.1 (sm_103a)"; }

// ---- single generator, 32-bit -------------------------------------------
int mtgp32_gpu_init(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para, uint32_t seed) {
    if (!para) return setErr(MTGP_ERR_INVALID, "null parameter set");
    Shape sh;
    int rc = checkParams<T32>(*para, &sh);
    if (rc) return rc;
    return initSeeded<T32>(out, para, seed);
}
int mtgp32_gpu_init_by_array(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para,
                             const uint32_t *array, int length) {
    if (!para || length < 0 || (length > 0 && !array))
        return setErr(MTGP_ERR_INVALID, "bad seed array");
    Shape sh;
    int rc = checkParams<T32>(*para, &sh);
    if (rc) return rc;
    return initKeyed<T32>(out, para, array, length);
}
int mtgp32_gpu_init_by_str(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para, const char *str) {
    if (!para || !str) return setErr(MTGP_ERR_INVALID, "bad seed string");
    Shape sh;
    int rc = checkParams<T32>(*para, &sh);
    if (rc) return rc;
    const std::vector<uint32_t> k = strKeys<T32>(str);
    return initKeyed<T32>(out, para, k.data(), (int)k.size());
}
void mtgp32_gpu_free(mtgp32_gpu_t *h) {
    if (!h) return;
    freeSingle(h);
}
int mtgp32_gpu_fill(mtgp32_gpu_t *h, int kind, void *out, size_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return fillSingle<T32>(h, kind, out, n, s);
}
int mtgp32_gpu_fill_uint32(mtgp32_gpu_t *h, uint32_t *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 0, o, n, s); }
int mtgp32_gpu_fill_close1_open2(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 1, o, n, s); }
int mtgp32_gpu_fill_close_open(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 2, o, n, s); }
int mtgp32_gpu_fill_open_close(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 3, o, n, s); }
int mtgp32_gpu_fill_open_open(mtgp32_gpu_t *h, float *o, size_t n, void *s) { return mtgp32_gpu_fill(h, 4, o, n, s); }
int mtgp32_gpu_skip(mtgp32_gpu_t *h, uint64_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return skipSingle(h->pool, n, s);
}
int mtgp32_gpu_fast_jump(mtgp32_gpu_t *h, const char *js, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.fastJump(0, js, s);
}
int mtgp32_gpu_jump_array(mtgp32_gpu_t *h, const uint32_t *p, int nw, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpArray(0, p, nw, s);
}
int mtgp32_gpu_jump_steps(mtgp32_gpu_t *h, uint64_t lo, uint64_t hi, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpSteps(0, lo, hi, s);
}
int mtgp32_gpu_export(mtgp32_gpu_t *h, mtgp32_fast_t *dst) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.exportTo(0, dst);
}
int mtgp32_gpu_import(mtgp32_gpu_t *h, const mtgp32_fast_t *src) { return importSingle<T32>(h, src); }
int mtgp32_gpu_get_window_host(mtgp32_gpu_t *h, uint32_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.getWindows(w, size < 0 ? 0 : (size_t)size);
}
int mtgp32_gpu_set_window_host(mtgp32_gpu_t *h, const uint32_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.setWindows(w, size < 0 ? 0 : (size_t)size);
}

// ---- single generator, 64-bit -------------------------------------------
int mtgp64_gpu_init(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para, uint64_t seed) {
    if (!para) return setErr(MTGP_ERR_INVALID, "null parameter set");
    Shape sh;
    int rc = checkParams<T64>(*para, &sh);
    if (rc) return rc;
    return initSeeded<T64>(out, para, seed);
}
int mtgp64_gpu_init_by_array(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para,
                             const uint64_t *array, int length) {
    if (!para || length < 0 || (length > 0 && !array))
        return setErr(MTGP_ERR_INVALID, "bad seed array");
    Shape sh;
    int rc = checkParams<T64>(*para, &sh);
    if (rc) return rc;
    return initKeyed<T64>(out, para, array, length);
}
int mtgp64_gpu_init_by_str(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para, const char *str) {
    if (!para || !str) return setErr(MTGP_ERR_INVALID, "bad seed string");
    Shape sh;
    int rc = checkParams<T64>(*para, &sh);
    if (rc) return rc;
    const std::vector<uint64_t> k = strKeys<T64>(str);
    return initKeyed<T64>(out, para, k.data(), (int)k.size());
}
void mtgp64_gpu_free(mtgp64_gpu_t *h) {
    if (!h) return;
    freeSingle(h);
}
int mtgp64_gpu_fill(mtgp64_gpu_t *h, int kind, void *out, size_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return fillSingle<T64>(h, kind, out, n, s);
}
int mtgp64_gpu_fill_uint64(mtgp64_gpu_t *h, uint64_t *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 0, o, n, s); }
int mtgp64_gpu_fill_close1_open2(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 1, o, n, s); }
int mtgp64_gpu_fill_close_open(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 2, o, n, s); }
int mtgp64_gpu_fill_open_close(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 3, o, n, s); }
int mtgp64_gpu_fill_open_open(mtgp64_gpu_t *h, double *o, size_t n, void *s) { return mtgp64_gpu_fill(h, 4, o, n, s); }
int mtgp64_gpu_skip(mtgp64_gpu_t *h, uint64_t n, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return skipSingle(h->pool, n, s);
}
int mtgp64_gpu_fast_jump(mtgp64_gpu_t *h, const char *js, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.fastJump(0, js, s);
}
int mtgp64_gpu_jump_array(mtgp64_gpu_t *h, const uint32_t *p, int nw, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpArray(0, p, nw, s);
}
int mtgp64_gpu_jump_steps(mtgp64_gpu_t *h, uint64_t lo, uint64_t hi, void *s) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.jumpSteps(0, lo, hi, s);
}
int mtgp64_gpu_export(mtgp64_gpu_t *h, mtgp64_fast_t *dst) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.exportTo(0, dst);
}
int mtgp64_gpu_import(mtgp64_gpu_t *h, const mtgp64_fast_t *src) { return importSingle<T64>(h, src); }
int mtgp64_gpu_get_window_host(mtgp64_gpu_t *h, uint64_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.getWindows(w, size < 0 ? 0 : (size_t)size);
}
int mtgp64_gpu_set_window_host(mtgp64_gpu_t *h, const uint64_t *w, int size) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null handle");
    return h->pool.setWindows(w, size < 0 ? 0 : (size_t)size);
}

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
        int up = uploadPlan(pl, s);
        if (!up) {
            const int pw = pl->bits == 32 ? static_cast<Pool<T32> *>(pl->pool)->polyWords()
                                          : static_cast<Pool<T64> *>(pl->pool)->polyWords();
            const int win = pl->bits == 32 ? static_cast<Pool<T32> *>(pl->pool)->tune.poly_window
                                           : static_cast<Pool<T64> *>(pl->pool)->tune.poly_window;
            up = powJobs(pl, pw, win, s);
        }
        if (!up) up = clearPrewin(pl, s);
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
    const int64_t v[8] = {pl->ntasks, pl->chunk, pl->bits == 64 ? 1 : pl->core, pl->grid,
                          pl->ntasks ? 1 + (pl->nstage > 0) + (pl->nparts > 0) +
                                           (pl->overlap && pl->nmain > 0)
                                     : 0,
                          pl->split ? 1 : 0, pl->npre, pl->overlap ? 1 : 0};
    for (int k = 0; k < n && k < 8; k++) values[k] = v[k];
    return MTGP_OK;
}

int mtgp_gpu_set_tuning(const char *key, int64_t value) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    Tuning t = g_tune_default;
    const int rc = applyTuning(t, key, value);
    if (!rc) g_tune_default = t;
    return rc;
}

int mtgp32_gpu_pool_set_tuning(mtgp32_gpu_pool_t *p, const char *key, int64_t value) {
    if (!p) return setErr(MTGP_ERR_INVALID, "null pool");
    return applyTuning(p->pool.tune, key, value);
}
int mtgp64_gpu_pool_set_tuning(mtgp64_gpu_pool_t *p, const char *key, int64_t value) {
    if (!p) return setErr(MTGP_ERR_INVALID, "null pool");
    return applyTuning(p->pool.tune, key, value);
}
int mtgp32_gpu_gen_set_tuning(mtgp32_gpu_t *h, const char *key, int64_t value) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null generator");
    return applyTuning(h->pool.tune, key, value);
}
int mtgp64_gpu_gen_set_tuning(mtgp64_gpu_t *h, const char *key, int64_t value) {
    if (!h) return setErr(MTGP_ERR_INVALID, "null generator");
    return applyTuning(h->pool.tune, key, value);
}

void mtgp_gpu_plan_free(mtgp_gpu_plan_t *pl) {
    if (!pl) return;
    cudaDeviceSynchronize();
    delete pl;
}

}  // extern "C"
