// host.cpp -- the C ABI of include/mtgp_gpu.h: error state, the allocation
// wrappers (with their test hook), the parameter conversion and the
// process-wide tuning defaults.  The other entry points live in plan.cpp
// (batched plans), single.cpp (single generators) and pool_api.cpp (pools
// and the autotuner).
//
// Host side of the GB300 MTGP generator: parameter validation, device memory
// for parameters and state windows, and the launches of the generation, jump
// and batched kernels.  Everything that produces random numbers runs on the
// GPU; there is no CPU generation path.
#include "host_internal.h"

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

namespace mtgp {
namespace host {

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

}  // namespace host
}  // namespace mtgp

int mtgp::recordError(int code, const char *msg) { return setErr(code, "%s", msg); }

extern "C" {

const char *mtgp_gpu_last_error(void) { return g_err.c_str(); }
const char *mtgp_gpu_version(void) { return "mtgp-gb300 0.1 (sm_103a)"; }

int mtgp_gpu_set_tuning(const char *key, int64_t value) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    Tuning t = g_tune_default;
    const int rc = applyTuning(t, key, value);
    if (!rc) g_tune_default = t;
    return rc;
}

}  // extern "C"
