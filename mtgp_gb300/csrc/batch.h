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
};

// grid <= 0: size the grid to the resident-CTA capacity of the GPU.
cudaError_t launchBatch32(int mexp, const DevParams32 *params, uint32_t *states,
                          const BatchTask *tasks, int ntasks, const BatchItem *items,
                          void *out, unsigned *counter, int grid, cudaStream_t s);
cudaError_t launchBatch64(int mexp, const DevParams64 *params, uint64_t *states,
                          const BatchTask *tasks, int ntasks, const BatchItem *items,
                          void *out, unsigned *counter, int grid, cudaStream_t s);

}  // namespace mtgp
