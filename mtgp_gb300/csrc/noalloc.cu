// noalloc.cu -- batched generation that allocates nothing.
//
// Callers that cannot allocate device memory use this entry point: engines
// whose device memory is all reserved up front in their own arena or under a
// hard budget, and plug-ins that may only use the buffers a host application
// hands them.  They pass the stream windows and the output buffer
// themselves; the descriptors
// the batched kernel needs (parameter sets, tasks, items and the work
// counter) go into one fixed-size array in device memory that is part of
// this library's image.
//
// Limits: at most kNaParams parameter sets and kNaItems work items per call
// (larger requests are rejected with MTGP_ERR_INVALID).  The array is shared
// by all calls in the process: each call overwrites it, so calls whose GPU
// work overlaps (different streams, or several host threads) race and must
// be serialised by the caller.  Every GPU that loads the library holds the
// array until the process exits.
//
// Each call waits for all work already queued on its stream before it
// launches (the descriptors are copied from host memory that must stay
// valid until the copies have read it, and the previous call's kernel may
// still be reading the array).  A stream that is being captured cannot be
// synchronised, so on such a stream the call returns MTGP_ERR_UNSUPPORTED
// and leaves the stream and its capture untouched.
#include <cstring>
#include <mutex>
#include <vector>

#include "batch.h"

namespace mtgp {
namespace {

constexpr int kNaParams = 16;
constexpr int kNaItems = 2048;
constexpr int kNaDevices = 64;

struct NaLayout {
    static constexpr size_t params = 0;
    static constexpr size_t tasks = params + sizeof(DevParams32) * kNaParams;
    static constexpr size_t items = tasks + sizeof(BatchTask) * kNaItems;
    static constexpr size_t counter = items + sizeof(BatchItem) * kNaItems;
    static constexpr size_t bytes = counter + 256;
};
static_assert(sizeof(DevParams32) % 16 == 0 && sizeof(BatchTask) % 16 == 0 &&
                  sizeof(BatchItem) % 8 == 0,
              "scratch fields must stay aligned");

// The scratch itself (about 116 KB).  In host code this name is only a
// stand-in for the symbol: its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_na_scratch[NaLayout::bytes];

std::mutex g_na_mu;
unsigned char *g_na_ptr[kNaDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device by the first call on it and kept for the life of the process (so
// the calls must not continue after a cudaDeviceReset of that device).
cudaError_t scratch(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNaDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess) return e;
        g_na_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_na_ptr[dev];
    return cudaSuccess;
}

int fail(int code, const char *msg) { return recordError(code, msg); }

}  // namespace
}  // namespace mtgp

using namespace mtgp;

extern "C" {

int mtgp32_gpu_batch_noalloc(const mtgp32_params_fast_t *params, int nparams,
                             const int *param_idx, uint32_t *dev_windows, int nstreams,
                             const mtgp_work_item_t *items, int nitems, void *dev_out,
                             void *stream) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!params || nparams <= 0 || !dev_windows || nstreams <= 0 || nitems < 0 ||
        (nitems > 0 && (!items || !dev_out)))
        return fail(MTGP_ERR_INVALID, "null or empty argument");
    if (nparams > kNaParams) return fail(MTGP_ERR_INVALID, "more than 16 parameter sets");
    if (nitems > kNaItems) return fail(MTGP_ERR_INVALID, "more than 2048 work items");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess)
        return fail(MTGP_ERR_CUDA, "cannot query the stream");
    if (cap != cudaStreamCaptureStatusNone)
        return fail(MTGP_ERR_UNSUPPORTED,
                    "the call synchronises its stream, which is being captured");
    Shape sh;
    if (!shape32(params[0].mexp, &sh)) return fail(MTGP_ERR_UNSUPPORTED, "exponent not supported");
    DevParams32 dp[kNaParams];
    for (int k = 0; k < nparams; k++) {
        if (params[k].mexp != sh.mexp) return fail(MTGP_ERR_INVALID, "parameter sets mix exponents");
        if (params[k].pos < 1 || params[k].pos > sh.n - sh.tn || params[k].sh1 < 0 ||
            params[k].sh1 > 31 || params[k].sh2 < 0 || params[k].sh2 > 31)
            return fail(MTGP_ERR_UNSUPPORTED, "parameter set outside the supported shape");
        toDev(params[k], &dp[k]);
    }
    // one task per stream; its items keep the caller's order
    std::vector<BatchTask> tasks;
    std::vector<BatchItem> bitems;
    std::vector<int> first(nstreams, -1), cnt(nstreams, 0);
    int mode = -3;
    for (int k = 0; k < nitems; k++) {
        const mtgp_work_item_t &it = items[k];
        if (it.stream >= (uint32_t)nstreams) return fail(MTGP_ERR_INVALID, "stream out of range");
        if (it.kind < -1 || it.kind > 4) return fail(MTGP_ERR_INVALID, "unknown output kind");
        if (it.kind >= 0 && it.out_offset % 4) return fail(MTGP_ERR_INVALID, "misaligned offset");
        if (it.skip) return fail(MTGP_ERR_INVALID, "skip is not supported here");
        if (it.count == 0) continue;
        mode = (mode == -3 || mode == it.kind) ? it.kind : -2;
        cnt[it.stream]++;
    }
    for (int st = 0, pos = 0; st < nstreams; st++) {
        first[st] = pos;
        pos += cnt[st];
    }
    bitems.resize((size_t)nitems);
    std::vector<int> fill(nstreams, 0);
    int used = 0;
    for (int k = 0; k < nitems; k++) {
        const mtgp_work_item_t &it = items[k];
        if (it.count == 0) continue;
        BatchItem &bi = bitems[(size_t)first[it.stream] + fill[it.stream]++];
        bi.out_off = it.out_offset;
        bi.count = it.count;
        bi.kind = it.kind;
        bi.pad_ = 0;
        used++;
    }
    for (int st = 0; st < nstreams; st++) {
        if (!cnt[st]) continue;
        BatchTask t{};
        t.stream = st;
        t.first = first[st];
        t.nitems = cnt[st];
        t.pidx = param_idx ? param_idx[st] : (nparams == nstreams ? st : 0);
        if (t.pidx < 0 || t.pidx >= nparams) return fail(MTGP_ERR_INVALID, "param_idx out of range");
        t.j0 = t.j1 = -1;
        t.wb = kWbStream;
        tasks.push_back(t);
    }
    if (tasks.empty()) return MTGP_OK;
    unsigned char *base = nullptr;
    cudaError_t e = scratch(&base);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + NaLayout::params, dp, sizeof(DevParams32) * nparams,
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + NaLayout::tasks, tasks.data(), sizeof(BatchTask) * tasks.size(),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + NaLayout::items, bitems.data(), sizeof(BatchItem) * used,
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        // the host vectors must stay valid until the copies have read them
        e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess) return fail(MTGP_ERR_CUDA, cudaGetErrorString(e));
    BatchLaunch b{};
    b.mexp = sh.mexp;
    b.mode = mode == -3 ? -1 : mode;
    b.grid = 0;
    b.core = b.mode == -2 ? 1 : 2;  // mixed kinds: the one-word core; else two words
    b.split = false;
    b.nwords = 0;
    b.polys = nullptr;
    b.tasks = reinterpret_cast<const BatchTask *>(base + NaLayout::tasks);
    b.ntasks = (int)tasks.size();
    b.items = reinterpret_cast<const BatchItem *>(base + NaLayout::items);
    b.out = dev_out;
    b.counter = reinterpret_cast<unsigned *>(base + NaLayout::counter);  // zeroed per launch
    b.stage = nullptr;
    b.stage_streams = nullptr;
    b.nstage = 0;
    e = launchBatch32(b, reinterpret_cast<const DevParams32 *>(base + NaLayout::params),
                      dev_windows, s);
    if (e != cudaSuccess) return fail(MTGP_ERR_CUDA, cudaGetErrorString(e));
    return MTGP_OK;
}

}  // extern "C"
