// batch_kernels.cu -- batched generation: many streams, uneven lengths, one
// persistent launch.
//
// A batch is a list of tasks; a task is one stream and a chain of work items
// (count, output kind, output byte offset) that continue that stream in
// order.  The grid is sized to the number of CTAs the GPU keeps resident;
// each CTA takes the next task from a device counter (tasks are sorted
// longest-first on the host, so the long ones start first), loads the
// stream's window into its shared ring, runs the items, and writes the
// advanced window back.  The arithmetic is the plain path's (run32/run64).
#include "batch.h"
#include "mtgp_device.cuh"

namespace mtgp {

namespace {

template <int N, int TN, int RING>
__global__ void __launch_bounds__(TN)
k_batch32(const DevParams32 *__restrict__ params, uint32_t *__restrict__ states,
          const BatchTask *__restrict__ tasks, int ntasks,
          const BatchItem *__restrict__ items, char *__restrict__ out,
          unsigned *__restrict__ counter) {
    __shared__ uint32_t ring[RING];
    __shared__ int s_task;
    constexpr uint32_t M = RING - 1;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        const BatchTask T = tasks[t];
        Lane32 L;
        L.load(params[T.pidx], threadIdx.x & 31);
        uint32_t *st = states + (size_t)T.stream * stateStride(N);
        for (int k = threadIdx.x; k < N; k += TN) ring[k] = st[k];
        __syncthreads();
        uint32_t phase = 0;
        for (int i = 0; i < T.nitems; i++) {
            const BatchItem I = items[T.first + i];
            char *o = out + I.out_off;
            switch (I.kind) {
            case 0: run32<N, TN, RING, 0>(ring, L, L.tmp, phase, I.count, (uint32_t *)o); break;
            case 1: run32<N, TN, RING, 1>(ring, L, L.flt, phase, I.count, (float *)o); break;
            case 2: run32<N, TN, RING, 2>(ring, L, L.flt, phase, I.count, (float *)o); break;
            case 3: run32<N, TN, RING, 3>(ring, L, L.flt, phase, I.count, (float *)o); break;
            case 4: run32<N, TN, RING, 4>(ring, L, L.flt, phase, I.count, (float *)o); break;
            default: run32<N, TN, RING, -1>(ring, L, L.tmp, phase, I.count, nullptr); break;
            }
            phase += (uint32_t)I.count;
        }
        for (int k = threadIdx.x; k < N; k += TN) st[k] = ring[(phase + k) & M];
        __syncthreads();
    }
}

template <int N, int TN, int RING>
__global__ void __launch_bounds__(TN)
k_batch64(const DevParams64 *__restrict__ params, uint64_t *__restrict__ states,
          const BatchTask *__restrict__ tasks, int ntasks,
          const BatchItem *__restrict__ items, char *__restrict__ out,
          unsigned *__restrict__ counter) {
    __shared__ uint64_t ring[RING];
    __shared__ int s_task;
    constexpr uint32_t M = RING - 1;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        const BatchTask T = tasks[t];
        Lane64 L;
        L.load(params[T.pidx], threadIdx.x & 31);
        uint64_t *st = states + (size_t)T.stream * stateStride(N);
        for (int k = threadIdx.x; k < N; k += TN) ring[k] = st[k];
        __syncthreads();
        uint32_t phase = 0;
        for (int i = 0; i < T.nitems; i++) {
            const BatchItem I = items[T.first + i];
            char *o = out + I.out_off;
            switch (I.kind) {
            case 0: run64<N, TN, RING, 0>(ring, L, L.tmp_lo, L.tmp_hi, phase, I.count, (uint64_t *)o); break;
            case 1: run64<N, TN, RING, 1>(ring, L, L.dbl_lo, L.dbl_hi, phase, I.count, (double *)o); break;
            case 2: run64<N, TN, RING, 2>(ring, L, L.dbl_lo, L.dbl_hi, phase, I.count, (double *)o); break;
            case 3: run64<N, TN, RING, 3>(ring, L, L.dbl_lo, L.dbl_hi, phase, I.count, (double *)o); break;
            case 4: run64<N, TN, RING, 4>(ring, L, L.dbl_lo, L.dbl_hi, phase, I.count, (double *)o); break;
            default: run64<N, TN, RING, -1>(ring, L, L.tmp_lo, L.tmp_hi, phase, I.count, nullptr); break;
            }
            phase += (uint32_t)I.count;
        }
        for (int k = threadIdx.x; k < N; k += TN) st[k] = ring[(phase + k) & M];
        __syncthreads();
    }
}

template <class K>
static cudaError_t occupancy(K kern, int tn, int *grid) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, tn, 0);
    if (e == cudaSuccess) *grid = sms * (per > 0 ? per : 1);
    return e;
}

template <int N, int TN, int RING>
static cudaError_t batch32(const DevParams32 *params, uint32_t *states, const BatchTask *tasks,
                           int ntasks, const BatchItem *items, char *out, unsigned *counter,
                           int grid, cudaStream_t s) {
    auto kern = k_batch32<N, TN, RING>;
    if (grid <= 0) {
        cudaError_t e = occupancy(kern, TN, &grid);
        if (e != cudaSuccess) return e;
    }
    if (grid > ntasks) grid = ntasks;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, TN, 0, s>>>(params, states, tasks, ntasks, items, out, counter);
    return cudaGetLastError();
}

template <int N, int TN, int RING>
static cudaError_t batch64(const DevParams64 *params, uint64_t *states, const BatchTask *tasks,
                           int ntasks, const BatchItem *items, char *out, unsigned *counter,
                           int grid, cudaStream_t s) {
    auto kern = k_batch64<N, TN, RING>;
    if (grid <= 0) {
        cudaError_t e = occupancy(kern, TN, &grid);
        if (e != cudaSuccess) return e;
    }
    if (grid > ntasks) grid = ntasks;
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, TN, 0, s>>>(params, states, tasks, ntasks, items, out, counter);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchBatch32(int mexp, const DevParams32 *params, uint32_t *states,
                          const BatchTask *tasks, int ntasks, const BatchItem *items,
                          void *out, unsigned *counter, int grid, cudaStream_t s) {
    if (ntasks <= 0) return cudaSuccess;
    char *o = static_cast<char *>(out);
    switch (mexp) {
    case 11213: return batch32<351, 256, 1024>(params, states, tasks, ntasks, items, o, counter, grid, s);
    case 23209: return batch32<726, 512, 2048>(params, states, tasks, ntasks, items, o, counter, grid, s);
    case 44497: return batch32<1391, 1024, 4096>(params, states, tasks, ntasks, items, o, counter, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launchBatch64(int mexp, const DevParams64 *params, uint64_t *states,
                          const BatchTask *tasks, int ntasks, const BatchItem *items,
                          void *out, unsigned *counter, int grid, cudaStream_t s) {
    if (ntasks <= 0) return cudaSuccess;
    char *o = static_cast<char *>(out);
    switch (mexp) {
    case 11213: return batch64<176, 128, 512>(params, states, tasks, ntasks, items, o, counter, grid, s);
    case 23209: return batch64<363, 256, 1024>(params, states, tasks, ntasks, items, o, counter, grid, s);
    case 44497: return batch64<696, 512, 2048>(params, states, tasks, ntasks, items, o, counter, grid, s);
    case 110503: return batch64<1727, 1024, 4096>(params, states, tasks, ntasks, items, o, counter, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace mtgp
