// batch_kernels.cu -- batched generation: many streams, uneven lengths, one
// persistent launch.
//
// A batch is a list of tasks; a task is one stream and a chain of work items
// (count, output kind, output byte offset) that continue that stream in
// order.  The grid is sized to the number of CTAs the GPU keeps resident;
// each CTA takes the next task from a device counter (tasks are sorted
// longest-first on the host, so the long ones start first), loads the
// stream's window into shared memory, runs the items with a generation core,
// and writes the advanced window back.
//
// Long requests are split into chunks that run on different CTAs: chunk c
// starts from the stream's window jumped ahead by its offset (X^off mod chi,
// applied inside the chunk's CTA with jump_device.cuh).  The jump is
// ALU-bound while generation is bound by the shared-memory data pipe, so the
// jumps of some CTAs overlap the generation of the others.  Only the last
// chunk keeps its final window, in a staging slot that k_unstage copies back
// after the launch, so no chunk can read a window that another chunk has
// already advanced.
//
// 32-bit streams run on the one-, two- or four-words-per-thread core
// (mtgp_device.cuh, mtgp_device4.cuh), two by default; plans whose items mix
// output kinds use the one-word core.
#include <mutex>
#include <vector>

#include "batch.h"
#include "jump_device.cuh"
#include "mtgp_device4.cuh"
#include "mtgp_device64x2.cuh"

namespace mtgp {

namespace {

// Jump geometry used inside the batched kernel (NT = the kernel's threads);
// the jump's shared buffers alias the generation buffer.
template <int N> struct SplitGeo32 { using G = void; };
template <> struct SplitGeo32<351> { using G = JGeo<351, 11, 256, 256, 2048>; };
template <> struct SplitGeo32<726> { using G = JGeo<726, 23, 512, 512, 4096>; };
template <int N> struct SplitGeo64 { using G = void; };
template <> struct SplitGeo64<176> { using G = JGeo<176, 7, 128, 128, 1024>; };
template <> struct SplitGeo64<363> { using G = JGeo<363, 13, 256, 256, 2048>; };

// Words per sub-step of the four-words-per-thread batched kernel (W/4
// threads per CTA).  It cannot exceed the shape's one-word-per-thread width
// TN: a sub-step's words are computed in parallel, so none of them may
// depend on another (y of word i is word i - N + pos, and pos <= N - TN).
template <int N, int TN> constexpr int kW4 = TN;

// Shared buffer (words) of the four-words-per-thread batched kernel: 3/4 of
// the shape's, so that 18 instead of 13 of its 64-thread CTAs fit an SM's
// shared memory (its registers allow 20); the window moves once per 10
// instead of 14 sub-steps.
template <int B> constexpr int kBuf4 = B / 4 * 3;

// The same for the K-words-per-thread kernels (NT = W/K threads).
template <int N, int K> struct SplitGeo32xK { using G = void; };
template <> struct SplitGeo32xK<351, 4> { using G = JGeo<351, 11, 64, 64, 1024>; };
template <> struct SplitGeo32xK<726, 4> { using G = JGeo<726, 23, 128, 128, 2048>; };
template <> struct SplitGeo32xK<351, 2> { using G = JGeo<351, 11, 128, 128, 1024>; };
template <> struct SplitGeo32xK<726, 2> { using G = JGeo<726, 23, 256, 256, 4096>; };

template <int N> constexpr bool kSplit32 = (N == 351 || N == 726);
template <int N> constexpr bool kSplit64 = (N == 176 || N == 363);

// Where a task's start window is: a pre-jumped window, or its stream's.
template <typename W>
__device__ __forceinline__ const W *startWindow(const BatchTask &T, const W *states,
                                                const W *prewin, int stride) {
    return T.pre > 0 ? prewin + (size_t)(T.pre - 1) * stride
                     : states + (size_t)T.stream * stride;
}

// The task's pre-jumped window, which each thread zeroes word by word right
// after reading it (so the slots are zero again for the next launch's jump
// parts, which XOR into them), or null.
template <typename W>
__device__ __forceinline__ W *preSlot(const BatchTask &T, W *prewin, int stride) {
    return T.pre > 0 ? prewin + (size_t)(T.pre - 1) * stride : nullptr;
}

template <typename W>
__device__ __forceinline__ W *endWindow(const BatchTask &T, W *states, W *stage, int stride) {
    return T.wb == kWbStream ? states + (size_t)T.stream * stride
         : T.wb >= 0         ? stage + (size_t)T.wb * stride
                             : nullptr;
}

// The task's start: the window jumped by polys[j0], then by polys[j1].
template <class Tr, class G>
__device__ __forceinline__ void jump_task(typename Tr::W *buf, const typename Tr::Lane &L,
                                          const BatchTask &T, const uint32_t *polys, int nwords) {
    const int j0 = T.j0, j1 = T.j1;
    jump_chain_impl<Tr, G, false>(
        buf, L, [=](int c) { return polys + (size_t)(c ? j1 : j0) * nwords; }, j1 >= 0 ? 2 : 1,
        nwords);
}

// The one-word kernels with mixed output kinds (MODE == -2) keep their
// generation buffer in dynamic shared memory and call each kind's loop out
// of line, addressing the buffer by this symbol (so the accesses stay
// shared-memory instructions).  Inlined together, the six loops' registers
// add up (63 instead of 32) and the resident CTAs halve.
extern __shared__ __align__(16) uint32_t g_mix32[];
extern __shared__ __align__(16) uint64_t g_mix64[];

// Resident CTAs that fix a mixed kernel's register budget: as many as its
// shared memory allows, at most `blocks`.
constexpr int mixBlocks(int blocks, size_t smem) {
    const int by_smem = (int)(204800 / smem) > 0 ? (int)(204800 / smem) : 1;
    return blocks < by_smem ? blocks : by_smem;
}

template <int N, int TN, int B, int KIND>
__device__ __noinline__ void mix32(Lane32 L, uint64_t n, char *o) {
    using OT = typename Out32<(KIND < 0 ? 0 : KIND)>::T;
    run32<N, TN, B, KIND>(g_mix32, L, L.otab(KIND < 0 ? 0 : KIND), n, (OT *)o);
}

template <int N, int W, int B, int KIND, int K>
__device__ __noinline__ void mixk32(Lane32 L, uint64_t n, char *o) {
    using C = CoreK<N, W, B, KIND, K>;
    C::run(g_mix32, L, L.otab(KIND < 0 ? 0 : KIND), n, (typename C::OT *)o);
}

template <int N, int TN, int B, int KIND>
__device__ __noinline__ void mix64(Lane64 L, uint64_t n, char *o) {
    using OT = typename Out64<(KIND < 0 ? 0 : KIND)>::T;
    run64<N, TN, B, KIND>(g_mix64, L, L.otab_lo(KIND < 0 ? 0 : KIND),
                          L.otab_hi(KIND < 0 ? 0 : KIND), n, (OT *)o);
}

// MODE >= -1: every item has output kind MODE (-1 = skip); MODE == -2:
// items of any kind (the kind is switched per item; dynamic shared memory of
// B words).  SPLIT: tasks may start with a jump.
template <int N, int TN, int B, int MODE, bool SPLIT>
__global__ void __launch_bounds__(TN, MODE == -2
                                         ? mixBlocks((SPLIT ? 1280 : 2048) / TN, sizeof(uint32_t) * B)
                                         : (SPLIT ? 1280 : 2048) / TN)
k_batch32(const DevParams32 *__restrict__ params, uint32_t *__restrict__ states,
          const BatchTask *__restrict__ tasks, int ntasks,
          const BatchItem *__restrict__ items, char *__restrict__ out,
          unsigned *__restrict__ counter, uint32_t *__restrict__ stage,
          const uint32_t *__restrict__ polys, int nwords, uint32_t *__restrict__ prewin) {
    __shared__ __align__(16) uint32_t sbuf[MODE == -2 ? 4 : B];
    uint32_t *const buf = MODE == -2 ? g_mix32 : sbuf;
    __shared__ int s_task;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        const BatchTask T = tasks[t];
        Lane32 L;
        L.load(params[T.pidx], threadIdx.x & 31);
        const uint32_t *st = startWindow(T, states, prewin, stateStride(N));
        uint32_t *clr = preSlot(T, prewin, stateStride(N));
        for (int k = threadIdx.x; k < N; k += TN) {
            buf[k] = st[k];
            if (clr) clr[k] = 0;
        }
        if constexpr (SPLIT && kSplit32<N>) {
            using G = typename SplitGeo32<N>::G;
            static_assert(G::NT == TN, "jump geometry must use the kernel's threads");
            static_assert(G::template bytes<uint32_t>(N / 32 + 1) <= sizeof(uint32_t) * B,
                          "jump buffers must fit the generation buffer");
            if (T.j0 >= 0) jump_task<Tr32, G>(buf, L, T, polys, nwords);
        }
        __syncthreads();
        for (int i = 0; i < T.nitems; i++) {
            const BatchItem I = items[T.first + i];
            char *o = out + I.out_off;
            if constexpr (MODE >= -1) {
                using OT = typename Out32<(MODE < 0 ? 0 : MODE)>::T;
                run32<N, TN, B, MODE>(buf, L, L.otab(MODE < 0 ? 0 : MODE), I.count, (OT *)o);
            } else {
                switch (I.kind) {
                case 0: mix32<N, TN, B, 0>(L, I.count, o); break;
                case 1: mix32<N, TN, B, 1>(L, I.count, o); break;
                case 2: mix32<N, TN, B, 2>(L, I.count, o); break;
                case 3: mix32<N, TN, B, 3>(L, I.count, o); break;
                case 4: mix32<N, TN, B, 4>(L, I.count, o); break;
                default: mix32<N, TN, B, -1>(L, I.count, nullptr); break;
                }
            }
        }
        uint32_t *dst = endWindow(T, states, stage, stateStride(N));
        if (dst)
            for (int k = threadIdx.x; k < N; k += TN) dst[k] = buf[k];
        __syncthreads();
    }
}

// K-words-per-thread core (W/K threads per CTA, K = 4 or 2).  SPLIT: tasks
// may start with a jump; the jump works on the window laid out linearly,
// which is then moved into the K planes of the generation buffer.  MODE ==
// -2: items of any kind, each kind's loop out of line on the generation
// buffer in dynamic shared memory, as in k_batch32.
template <int N, int W, int B, int MODE, bool SPLIT, int K>
__global__ void __launch_bounds__(W / K,
                                  MODE == -2
                                      ? mixBlocks(1280 * K / W,
                                                  sizeof(uint32_t) * GeoK<N, W, B, K>::BUF)
                                      : 1280 * K / W)
k_batch32xk(const DevParams32 *__restrict__ params, uint32_t *__restrict__ states,
            const BatchTask *__restrict__ tasks, int ntasks,
            const BatchItem *__restrict__ items, char *__restrict__ out,
            unsigned *__restrict__ counter, uint32_t *__restrict__ stage,
            const uint32_t *__restrict__ polys, int nwords,
            uint32_t *__restrict__ prewin) {
    constexpr int T = W / K;
    constexpr int PW = GeoK<N, W, B, K>::PW;
    constexpr int BUF = GeoK<N, W, B, K>::BUF;
    __shared__ __align__(16) uint32_t sbuf[MODE == -2 ? 4 : BUF];
    uint32_t *const buf = MODE == -2 ? g_mix32 : sbuf;
    __shared__ int s_task;
    (void)polys;
    (void)nwords;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        const BatchTask TK = tasks[t];
        Lane32 L;
        L.load(params[TK.pidx], threadIdx.x & 31);
        const uint32_t *src = startWindow(TK, states, prewin, stateStride(N));
        bool planar = true;
        if constexpr (SPLIT && kSplit32<N>) {
            using G = typename SplitGeo32xK<N, K>::G;
            static_assert(G::NT == T, "jump geometry must use the kernel's threads");
            static_assert(G::template bytes<uint32_t>(N / 32 + 1) <= sizeof(uint32_t) * BUF,
                          "jump buffers must fit the generation buffer");
            if (TK.j0 >= 0) {
                for (int k = threadIdx.x; k < N; k += T) buf[k] = src[k];
                jump_task<Tr32, G>(buf, L, TK, polys, nwords);  // ends with a barrier
                constexpr int PER = (N + T - 1) / T;
                uint32_t v[PER];
#pragma unroll
                for (int i = 0; i < PER; i++) {
                    const int k = threadIdx.x + i * T;
                    if (k < N) v[i] = buf[k];
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < PER; i++) {
                    const int k = threadIdx.x + i * T;
                    if (k < N) buf[plane_at<PW, K>(k)] = v[i];
                }
                planar = false;
            }
        }
        if (planar) {
            uint32_t *clr = preSlot(TK, prewin, stateStride(N));
            for (int k = threadIdx.x; k < N; k += T) {
                buf[plane_at<PW, K>(k)] = src[k];
                if (clr) clr[k] = 0;
            }
        }
        __syncthreads();
        for (int i = 0; i < TK.nitems; i++) {
            const BatchItem I = items[TK.first + i];
            char *o = out + I.out_off;
            if constexpr (MODE >= -1) {
                using C = CoreK<N, W, B, MODE, K>;
                C::run(buf, L, L.otab(MODE < 0 ? 0 : MODE), I.count, (typename C::OT *)o);
            } else {
                switch (I.kind) {
                case 0: mixk32<N, W, B, 0, K>(L, I.count, o); break;
                case 1: mixk32<N, W, B, 1, K>(L, I.count, o); break;
                case 2: mixk32<N, W, B, 2, K>(L, I.count, o); break;
                case 3: mixk32<N, W, B, 3, K>(L, I.count, o); break;
                case 4: mixk32<N, W, B, 4, K>(L, I.count, o); break;
                default: mixk32<N, W, B, -1, K>(L, I.count, nullptr); break;
                }
            }
        }
        uint32_t *dst = endWindow(TK, states, stage, stateStride(N));
        if (dst)
            for (int k = threadIdx.x; k < N; k += T) dst[k] = buf[plane_at<PW, K>(k)];
        __syncthreads();
    }
}

template <int N, int TN, int B, int MODE, bool SPLIT>
__global__ void __launch_bounds__(TN, MODE == -2
                                         ? mixBlocks((SPLIT ? 1280 : 2048) / TN, sizeof(uint64_t) * B)
                                         : (SPLIT ? 1280 : 2048) / TN)
k_batch64(const DevParams64 *__restrict__ params, uint64_t *__restrict__ states,
          const BatchTask *__restrict__ tasks, int ntasks,
          const BatchItem *__restrict__ items, char *__restrict__ out,
          unsigned *__restrict__ counter, uint64_t *__restrict__ stage,
          const uint32_t *__restrict__ polys, int nwords, uint64_t *__restrict__ prewin) {
    __shared__ __align__(16) uint64_t sbuf[MODE == -2 ? 4 : B];
    uint64_t *const buf = MODE == -2 ? g_mix64 : sbuf;
    __shared__ int s_task;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        const BatchTask T = tasks[t];
        Lane64 L;
        L.load(params[T.pidx], threadIdx.x & 31);
        const uint64_t *st = startWindow(T, states, prewin, stateStride(N));
        uint64_t *clr = preSlot(T, prewin, stateStride(N));
        for (int k = threadIdx.x; k < N; k += TN) {
            buf[k] = st[k];
            if (clr) clr[k] = 0;
        }
        if constexpr (SPLIT && kSplit64<N>) {
            using G = typename SplitGeo64<N>::G;
            static_assert(G::NT == TN, "jump geometry must use the kernel's threads");
            static_assert(G::template bytes<uint64_t>(N * 2) <= sizeof(uint64_t) * B,
                          "jump buffers must fit the generation buffer");
            if (T.j0 >= 0) jump_task<Tr64, G>(buf, L, T, polys, nwords);
        }
        __syncthreads();
        for (int i = 0; i < T.nitems; i++) {
            const BatchItem I = items[T.first + i];
            char *o = out + I.out_off;
            if constexpr (MODE >= -1) {
                using OT = typename Out64<(MODE < 0 ? 0 : MODE)>::T;
                run64<N, TN, B, MODE>(buf, L, L.otab_lo(MODE < 0 ? 0 : MODE),
                                      L.otab_hi(MODE < 0 ? 0 : MODE), I.count, (OT *)o);
            } else {
                switch (I.kind) {
                case 0: mix64<N, TN, B, 0>(L, I.count, o); break;
                case 1: mix64<N, TN, B, 1>(L, I.count, o); break;
                case 2: mix64<N, TN, B, 2>(L, I.count, o); break;
                case 3: mix64<N, TN, B, 3>(L, I.count, o); break;
                case 4: mix64<N, TN, B, 4>(L, I.count, o); break;
                default: mix64<N, TN, B, -1>(L, I.count, nullptr); break;
                }
            }
        }
        uint64_t *dst = endWindow(T, states, stage, stateStride(N));
        if (dst)
            for (int k = threadIdx.x; k < N; k += TN) dst[k] = buf[k];
        __syncthreads();
    }
}

// 64-bit two-words-per-thread core (W/2 threads per CTA): items of one
// output kind (MODE >= -1), tasks that start from the stream's window or a
// window jumped ahead of the launch (no jump code: plans on this core make
// every jumped start ahead of the launch).
template <int N, int W, int B, int MODE>
__global__ void __launch_bounds__(W / 2)
k_batch64x2(const DevParams64 *__restrict__ params, uint64_t *__restrict__ states,
            const BatchTask *__restrict__ tasks, int ntasks,
            const BatchItem *__restrict__ items, char *__restrict__ out,
            unsigned *__restrict__ counter, uint64_t *__restrict__ stage,
            const uint32_t *__restrict__ polys, int nwords, uint64_t *__restrict__ prewin) {
    using C = Core64x2<N, W, B, MODE>;
    constexpr int T = W / 2;
    __shared__ __align__(16) uint64_t buf[C::G::BUF];
    __shared__ int s_task;
    (void)polys;
    (void)nwords;
    for (;;) {
        if (threadIdx.x == 0) s_task = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        const BatchTask TK = tasks[t];
        Lane64 L;
        L.load(params[TK.pidx], threadIdx.x & 31);
        const uint64_t *src = startWindow(TK, states, prewin, stateStride(N));
        uint64_t *clr = preSlot(TK, prewin, stateStride(N));
        for (int k = threadIdx.x; k < N; k += T) {
            buf[C::at(k)] = src[k];
            if (clr) clr[k] = 0;
        }
        __syncthreads();
        for (int i = 0; i < TK.nitems; i++) {
            const BatchItem I = items[TK.first + i];
            C::run(buf, L, L.otab_lo(MODE < 0 ? 0 : MODE), L.otab_hi(MODE < 0 ? 0 : MODE),
                   I.count, (typename C::OT *)(out + I.out_off));
        }
        uint64_t *dst = endWindow(TK, states, stage, stateStride(N));
        if (dst)
            for (int k = threadIdx.x; k < N; k += T) dst[k] = buf[C::at(k)];
        __syncthreads();
    }
}

// Staged windows back to their streams: block k copies slot k.
template <typename W, int N>
__global__ void k_unstage(W *__restrict__ states, const W *__restrict__ stage,
                          const int32_t *__restrict__ streams) {
    const W *src = stage + (size_t)blockIdx.x * stateStride(N);
    W *dst = states + (size_t)streams[blockIdx.x] * stateStride(N);
    for (int k = threadIdx.x; k < N; k += blockDim.x) dst[k] = src[k];
}

// Resident CTAs of a kernel on the current device (cached per kernel and
// device: the occupancy query is not free and servers launch often).
template <class K>
static cudaError_t resident(K kern, int tn, int *grid, size_t smem = 0) {
    struct Entry {
        const void *fn;
        int dev, tn, grid;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const void *fn = reinterpret_cast<const void *>(kern);
    {
        std::lock_guard<std::mutex> lk(mu);
        for (const Entry &c : cache)
            if (c.fn == fn && c.dev == dev && c.tn == tn) {
                *grid = c.grid;
                return cudaSuccess;
            }
    }
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, tn, smem);
    if (e != cudaSuccess) return e;
    *grid = sms * (per > 0 ? per : 1);
    std::lock_guard<std::mutex> lk(mu);
    cache.push_back({fn, dev, tn, *grid});
    return cudaSuccess;
}

// work counter reset -> persistent kernel
template <typename W, class K, class P>
static cudaError_t go(K kern, int tn, const BatchLaunch &b, const P *params, W *states,
                      cudaStream_t s, size_t smem = 0) {
    int grid = b.grid;
    if (grid <= 0) {
        cudaError_t e = resident(kern, tn, &grid, smem);
        if (e != cudaSuccess) return e;
    }
    if (grid > b.ntasks) grid = b.ntasks;
    cudaError_t e = cudaMemsetAsync(b.counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    kern<<<grid, tn, smem, s>>>(params, states, b.tasks, b.ntasks, b.items,
                             static_cast<char *>(b.out), b.counter, static_cast<W *>(b.stage),
                             b.polys, b.nwords, static_cast<W *>(b.prewin));
    return cudaGetLastError();
}

template <int N, int TN, int B, bool SPLIT>
static cudaError_t mode32(const BatchLaunch &b, const DevParams32 *p, uint32_t *st,
                          cudaStream_t s) {
    switch (b.mode) {
    case -1: return go<uint32_t>(k_batch32<N, TN, B, -1, SPLIT>, TN, b, p, st, s);
    case 0: return go<uint32_t>(k_batch32<N, TN, B, 0, SPLIT>, TN, b, p, st, s);
    case 1: return go<uint32_t>(k_batch32<N, TN, B, 1, SPLIT>, TN, b, p, st, s);
    case 2: return go<uint32_t>(k_batch32<N, TN, B, 2, SPLIT>, TN, b, p, st, s);
    case 3: return go<uint32_t>(k_batch32<N, TN, B, 3, SPLIT>, TN, b, p, st, s);
    case 4: return go<uint32_t>(k_batch32<N, TN, B, 4, SPLIT>, TN, b, p, st, s);
    default:
        return go<uint32_t>(k_batch32<N, TN, B, -2, SPLIT>, TN, b, p, st, s,
                            sizeof(uint32_t) * B);
    }
}

template <int N, int W, int B, bool SPLIT, int K>
static cudaError_t mode32xk(const BatchLaunch &b, const DevParams32 *p, uint32_t *st,
                            cudaStream_t s) {
    constexpr int T = W / K;
    switch (b.mode) {
    case -1: return go<uint32_t>(k_batch32xk<N, W, B, -1, SPLIT, K>, T, b, p, st, s);
    case 0: return go<uint32_t>(k_batch32xk<N, W, B, 0, SPLIT, K>, T, b, p, st, s);
    case 1: return go<uint32_t>(k_batch32xk<N, W, B, 1, SPLIT, K>, T, b, p, st, s);
    case 2: return go<uint32_t>(k_batch32xk<N, W, B, 2, SPLIT, K>, T, b, p, st, s);
    case 3: return go<uint32_t>(k_batch32xk<N, W, B, 3, SPLIT, K>, T, b, p, st, s);
    case 4: return go<uint32_t>(k_batch32xk<N, W, B, 4, SPLIT, K>, T, b, p, st, s);
    default:
        return go<uint32_t>(k_batch32xk<N, W, B, -2, SPLIT, K>, T, b, p, st, s,
                            sizeof(uint32_t) * GeoK<N, W, B, K>::BUF);
    }
}

template <int N, int TN, int B, bool SPLIT>
static cudaError_t mode64(const BatchLaunch &b, const DevParams64 *p, uint64_t *st,
                          cudaStream_t s) {
    switch (b.mode) {
    case -1: return go<uint64_t>(k_batch64<N, TN, B, -1, SPLIT>, TN, b, p, st, s);
    case 0: return go<uint64_t>(k_batch64<N, TN, B, 0, SPLIT>, TN, b, p, st, s);
    case 1: return go<uint64_t>(k_batch64<N, TN, B, 1, SPLIT>, TN, b, p, st, s);
    case 2: return go<uint64_t>(k_batch64<N, TN, B, 2, SPLIT>, TN, b, p, st, s);
    case 3: return go<uint64_t>(k_batch64<N, TN, B, 3, SPLIT>, TN, b, p, st, s);
    case 4: return go<uint64_t>(k_batch64<N, TN, B, 4, SPLIT>, TN, b, p, st, s);
    default:
        return go<uint64_t>(k_batch64<N, TN, B, -2, SPLIT>, TN, b, p, st, s,
                            sizeof(uint64_t) * B);
    }
}

template <int N, int TN, int B>
static cudaError_t run32x(const BatchLaunch &b, const DevParams32 *p, uint32_t *st,
                          cudaStream_t s) {
    cudaError_t e;
    constexpr int W = kW4<N, TN>;
    if (b.split) {
        if constexpr (kSplit32<N>)
            e = b.core == 4   ? mode32xk<N, W, kBuf4<B>, true, 4>(b, p, st, s)
                : b.core == 2 ? mode32xk<N, W, B, true, 2>(b, p, st, s)
                              : mode32<N, TN, B, true>(b, p, st, s);
        else
            return cudaErrorInvalidValue;
    } else if (b.core == 4) {
        e = mode32xk<N, W, kBuf4<B>, false, 4>(b, p, st, s);
    } else if (b.core == 2) {
        e = mode32xk<N, W, B, false, 2>(b, p, st, s);
    } else {
        e = mode32<N, TN, B, false>(b, p, st, s);
    }
    if (e != cudaSuccess || b.nstage <= 0) return e;
    k_unstage<uint32_t, N><<<b.nstage, 128, 0, s>>>(st, static_cast<const uint32_t *>(b.stage),
                                                    b.stage_streams);
    return cudaGetLastError();
}

template <int N, int W, int B>
static cudaError_t mode64x2(const BatchLaunch &b, const DevParams64 *p, uint64_t *st,
                            cudaStream_t s) {
    constexpr int T = W / 2;
    switch (b.mode) {
    case -1: return go<uint64_t>(k_batch64x2<N, W, B, -1>, T, b, p, st, s);
    case 0: return go<uint64_t>(k_batch64x2<N, W, B, 0>, T, b, p, st, s);
    case 1: return go<uint64_t>(k_batch64x2<N, W, B, 1>, T, b, p, st, s);
    case 2: return go<uint64_t>(k_batch64x2<N, W, B, 2>, T, b, p, st, s);
    case 3: return go<uint64_t>(k_batch64x2<N, W, B, 3>, T, b, p, st, s);
    case 4: return go<uint64_t>(k_batch64x2<N, W, B, 4>, T, b, p, st, s);
    default: return cudaErrorInvalidValue;  // mixed kinds run on the one-word core
    }
}

template <int N, int TN, int B>
static cudaError_t run64x(const BatchLaunch &b, const DevParams64 *p, uint64_t *st,
                          cudaStream_t s) {
    cudaError_t e;
    if (b.core != 1 && !b.split && b.mode != -2) {
        e = mode64x2<N, TN, B>(b, p, st, s);
    } else if (b.split) {
        if constexpr (kSplit64<N>) e = mode64<N, TN, B, true>(b, p, st, s);
        else return cudaErrorInvalidValue;
    } else {
        e = mode64<N, TN, B, false>(b, p, st, s);
    }
    if (e != cudaSuccess || b.nstage <= 0) return e;
    k_unstage<uint64_t, N><<<b.nstage, 128, 0, s>>>(st, static_cast<const uint64_t *>(b.stage),
                                                    b.stage_streams);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchBatch32(const BatchLaunch &b, const DevParams32 *params, uint32_t *states,
                          cudaStream_t s) {
    if (b.ntasks <= 0) return cudaSuccess;
#define X(M, N, T, B) \
    if (b.mexp == M) return run32x<N, T, B>(b, params, states, s);
    MTGP_SHAPES32(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchBatch64(const BatchLaunch &b, const DevParams64 *params, uint64_t *states,
                          cudaStream_t s) {
    if (b.ntasks <= 0) return cudaSuccess;
#define X(M, N, T, B) \
    if (b.mexp == M) return run64x<N, T, B>(b, params, states, s);
    MTGP_SHAPES64(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchUnstage32(int mexp, uint32_t *states, const void *stage,
                            const int32_t *streams, int nstage, cudaStream_t s) {
    if (nstage <= 0) return cudaSuccess;
#define X(M, N, T, B)                                                                       \
    if (mexp == M) {                                                                        \
        k_unstage<uint32_t, N><<<nstage, 128, 0, s>>>(                                      \
            states, static_cast<const uint32_t *>(stage), streams);                         \
        return cudaGetLastError();                                                          \
    }
    MTGP_SHAPES32(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchUnstage64(int mexp, uint64_t *states, const void *stage,
                            const int32_t *streams, int nstage, cudaStream_t s) {
    if (nstage <= 0) return cudaSuccess;
#define X(M, N, T, B)                                                                       \
    if (mexp == M) {                                                                        \
        k_unstage<uint64_t, N><<<nstage, 128, 0, s>>>(                                      \
            states, static_cast<const uint64_t *>(stage), streams);                         \
        return cudaGetLastError();                                                          \
    }
    MTGP_SHAPES64(X)
#undef X
    return cudaErrorInvalidValue;
}

bool batchSplits32(int mexp) { return mexp == 11213 || mexp == 23209; }
bool batchSplits64(int mexp) { return mexp == 11213 || mexp == 23209; }

// Resident CTAs of the kernel a plan with (or without) split requests uses
// with the given generation core.
template <int N, int T, int B>
static int resident32(bool split, int core) {
    int g = 0;
    const bool jumps = split && kSplit32<N>;
    constexpr int W = kW4<N, T>;
    if (core == 4) {
        if (jumps) resident(k_batch32xk<N, W, kBuf4<B>, 0, kSplit32<N>, 4>, W / 4, &g);
        else resident(k_batch32xk<N, W, kBuf4<B>, 0, false, 4>, W / 4, &g);
    } else if (core == 2) {
        if (jumps) resident(k_batch32xk<N, W, B, 0, kSplit32<N>, 2>, W / 2, &g);
        else resident(k_batch32xk<N, W, B, 0, false, 2>, W / 2, &g);
    } else {
        if (jumps) resident(k_batch32<N, T, B, 0, kSplit32<N>>, T, &g);
        else resident(k_batch32<N, T, B, 0, false>, T, &g);
    }
    return g;
}

int batchResident32(int mexp, bool split, int core) {
#define X(M, N, T, B) \
    if (mexp == M) return resident32<N, T, B>(split, core);
    MTGP_SHAPES32(X)
#undef X
    return 0;
}

int batchResident64(int mexp, bool split, int core) {
    int g = 0;
#define X(M, N, T, B) \
    if (mexp == M) {                                                  \
        if (core != 1 && !split) resident(k_batch64x2<N, T, B, 0>, T / 2, &g); \
        else if (split) resident(k_batch64<N, T, B, 0, true>, T, &g);  \
        else resident(k_batch64<N, T, B, 0, false>, T, &g);           \
    }
    MTGP_SHAPES64(X)
#undef X
    return g;
}

}  // namespace mtgp
