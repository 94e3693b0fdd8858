// batch.h -- device descriptors of a batched launch (batch_kernels.cu).
#pragma once
#include <cstdint>

#include "internal.h"

namespace mtgp {

struct BatchItem {
    uint64_t out_off;  // byte offset of the first value in the output buffer
    uint64_t count;    // values to produce
    int32_t kind;      // MTGP_KIND_*, or -1 = advance without output
    int32_t pad_;
};

struct BatchTask {
    int32_t stream;    // stream index in the pool
    int32_t first;     // first item (items of one task are consecutive)
    int32_t nitems;
    int32_t pidx;      // parameter-set index of the stream
    // The task starts from the stream's window jumped by polynomial j0,
    // then by j1 (indices into BatchLaunch::polys, uint32-array form;
    // -1 = none): a task that starts later in the stream than the window.
    int32_t j0, j1;
    // Where the advanced window goes: kWbStream = back to the stream,
    // kWbNone = nowhere (a task that is not the stream's last), k >= 0 =
    // staging slot k (the last task of a stream with several; copied to the
    // stream after the launch, so no task can read a window that another
    // task already advanced).
    int32_t wb;
    // k + 1: the task starts from pre-jumped window k (BatchLaunch::prewin,
    // made before the launch by jump parts) instead of the stream's window;
    // 0: from the stream's window
    int32_t pre;
};
static_assert(sizeof(BatchTask) == 32, "BatchTask is 32 bytes");
constexpr int32_t kWbStream = -1;
constexpr int32_t kWbNone = -2;

// grid <= 0: size the grid to the resident-CTA capacity of the GPU.
// mode: the output kind shared by every item (-1 = all skips), or -2 when
// items mix kinds.
// One batched launch.  split: some tasks start with a jump (the kernel
// variant with the jump code runs).  After the kernel, staged final windows
// (stage slot k -> stream stage_streams[k]) are copied back.
struct BatchLaunch {
    int mexp, mode, grid;
    int core;                       // 32-bit generation core: 1, 2 or 4 words per thread
    bool split;
    int nwords;                     // words of every jump polynomial
    const uint32_t *polys;          // jump polynomials, nwords words each
    const BatchTask *tasks;
    int ntasks;
    const BatchItem *items;
    void *out;
    unsigned *counter;
    void *stage;
    const int32_t *stage_streams;
    int nstage;
    void *prewin;                   // pre-jumped start windows (BatchTask::pre);
                                    // zero on entry, zeroed again as tasks read them
};
cudaError_t launchBatch32(const BatchLaunch &b, const DevParams32 *params, uint32_t *states,
                          cudaStream_t s);
cudaError_t launchBatch64(const BatchLaunch &b, const DevParams64 *params, uint64_t *states,
                          cudaStream_t s);
// Staged final windows back to their streams (the copy launchBatch runs
// after its kernel when nstage > 0), on its own.
cudaError_t launchUnstage32(int mexp, uint32_t *states, const void *stage,
                            const int32_t *streams, int nstage, cudaStream_t s);
cudaError_t launchUnstage64(int mexp, uint64_t *states, const void *stage,
                            const int32_t *streams, int nstage, cudaStream_t s);
// Number of CTAs of the batched kernel resident at once on the device
// (32-bit: for the given generation core, 1, 2 or 4).
int batchResident32(int mexp, bool split, int core);
int batchResident64(int mexp, bool split, int core = 1);
// Whether split requests are supported for this exponent.
bool batchSplits32(int mexp);
bool batchSplits64(int mexp);

}  // namespace mtgp
