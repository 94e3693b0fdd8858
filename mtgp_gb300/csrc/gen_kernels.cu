// gen_kernels.cu -- plain generation: one CTA per generator.
//
// This is the shape of the reference's CUDA sample kernels
// (cuda-sample/mtgp32-cuda.cu:171-297, mtgp64-cuda.cu:208-392): a CTA loads
// its generator's window from HBM into a shared ring, emits n outputs, and
// writes the advanced window back.  Unlike the sample it accepts any n (not
// a multiple of 3*TN), any parameter set per CTA, all five output kinds and
// every Mersenne exponent of the reference's tables.
#include "mtgp_device64x2.cuh"

namespace mtgp {

bool shape32(int mexp, Shape *s) {
#define X(M, N, T, B) \
    if (mexp == M) { *s = {M, N, T, B}; return true; }
    MTGP_SHAPES32(X)
#undef X
    return false;
}

bool shape64(int mexp, Shape *s) {
#define X(M, N, T, B) \
    if (mexp == M) { *s = {M, N, T, B}; return true; }
    MTGP_SHAPES64(X)
#undef X
    return false;
}

template <int N, int TN, int B, int KIND>
__global__ void __launch_bounds__(TN)
k_gen32(const DevParams32 *__restrict__ params, const int *__restrict__ pidx,
        uint32_t *__restrict__ states, void *__restrict__ out, uint64_t n,
        uint64_t out_stride) {
    __shared__ uint32_t ring[B];
    const int g = blockIdx.x;
    const DevParams32 &P = params[pidx ? pidx[g] : g];
    Lane32 L;
    L.load(P, threadIdx.x & 31);
    uint32_t *st = states + (size_t)g * stateStride(N);
    for (int k = threadIdx.x; k < N; k += TN) ring[k] = st[k];
    __syncthreads();
    using T = typename Out32<(KIND < 0 ? 0 : KIND)>::T;
    T *o = KIND < 0 ? nullptr : reinterpret_cast<T *>(out) + (size_t)g * out_stride;
    run32<N, TN, B, KIND>(ring, L, L.otab(KIND < 0 ? 0 : KIND), n, o);
    for (int k = threadIdx.x; k < N; k += TN) st[k] = ring[k];
}

// Same as k_gen32 with the K-words-per-thread core (W = parallel width, W/K
// threads per CTA, K = 4 or 2).
template <int N, int W, int B, int KIND, int K>
__global__ void __launch_bounds__(W / K)
k_gen32xk(const DevParams32 *__restrict__ params, const int *__restrict__ pidx,
          uint32_t *__restrict__ states, void *__restrict__ out, uint64_t n,
          uint64_t out_stride) {
    using C = CoreK<N, W, B, KIND, K>;
    __shared__ __align__(16) uint32_t buf[GeoK<N, W, B, K>::BUF];
    const int g = blockIdx.x;
    const DevParams32 &P = params[pidx ? pidx[g] : g];
    Lane32 L;
    L.load(P, threadIdx.x & 31);
    uint32_t *st = states + (size_t)g * stateStride(N);
    for (int k = threadIdx.x; k < N; k += W / K) buf[plane_at<C::G::PW, K>(k)] = st[k];
    __syncthreads();
    using T = typename C::OT;
    T *o = KIND < 0 ? nullptr : reinterpret_cast<T *>(out) + (size_t)g * out_stride;
    C::run(buf, L, L.otab(KIND < 0 ? 0 : KIND), n, o);
    for (int k = threadIdx.x; k < N; k += W / K) st[k] = buf[plane_at<C::G::PW, K>(k)];
}

template <int N, int W, int B, int K>
static cudaError_t gen32xk(int kind, const DevParams32 *params, const int *pidx,
                           uint32_t *states, int ngen, void *out, uint64_t n, uint64_t os,
                           cudaStream_t s) {
    dim3 grid(ngen), b(W / K);
    switch (kind) {
    case -1: k_gen32xk<N, W, B, -1, K><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 0: k_gen32xk<N, W, B, 0, K><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 1: k_gen32xk<N, W, B, 1, K><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 2: k_gen32xk<N, W, B, 2, K><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 3: k_gen32xk<N, W, B, 3, K><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 4: k_gen32xk<N, W, B, 4, K><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int N, int TN, int B, int KIND>
__global__ void __launch_bounds__(TN)
k_gen64(const DevParams64 *__restrict__ params, const int *__restrict__ pidx,
        uint64_t *__restrict__ states, void *__restrict__ out, uint64_t n,
        uint64_t out_stride) {
    __shared__ uint64_t ring[B];
    const int g = blockIdx.x;
    const DevParams64 &P = params[pidx ? pidx[g] : g];
    Lane64 L;
    L.load(P, threadIdx.x & 31);
    uint64_t *st = states + (size_t)g * stateStride(N);
    for (int k = threadIdx.x; k < N; k += TN) ring[k] = st[k];
    __syncthreads();
    using T = typename Out64<(KIND < 0 ? 0 : KIND)>::T;
    T *o = KIND < 0 ? nullptr : reinterpret_cast<T *>(out) + (size_t)g * out_stride;
    run64<N, TN, B, KIND>(ring, L, L.otab_lo(KIND < 0 ? 0 : KIND),
                          L.otab_hi(KIND < 0 ? 0 : KIND), n, o);
    for (int k = threadIdx.x; k < N; k += TN) st[k] = ring[k];
}

// Same as k_gen64 with the two-words-per-thread core (W/2 threads per CTA).
template <int N, int W, int B, int KIND>
__global__ void __launch_bounds__(W / 2)
k_gen64x2(const DevParams64 *__restrict__ params, const int *__restrict__ pidx,
          uint64_t *__restrict__ states, void *__restrict__ out, uint64_t n,
          uint64_t out_stride) {
    using C = Core64x2<N, W, B, KIND>;
    __shared__ __align__(16) uint64_t buf[C::G::BUF];
    const int g = blockIdx.x;
    const DevParams64 &P = params[pidx ? pidx[g] : g];
    Lane64 L;
    L.load(P, threadIdx.x & 31);
    uint64_t *st = states + (size_t)g * stateStride(N);
    for (int k = threadIdx.x; k < N; k += W / 2) buf[C::at(k)] = st[k];
    __syncthreads();
    using T = typename C::OT;
    T *o = KIND < 0 ? nullptr : reinterpret_cast<T *>(out) + (size_t)g * out_stride;
    C::run(buf, L, L.otab_lo(KIND < 0 ? 0 : KIND), L.otab_hi(KIND < 0 ? 0 : KIND), n, o);
    for (int k = threadIdx.x; k < N; k += W / 2) st[k] = buf[C::at(k)];
}

template <int N, int W, int B>
static cudaError_t gen64x2(int kind, const DevParams64 *params, const int *pidx,
                           uint64_t *states, int ngen, void *out, uint64_t n, uint64_t os,
                           cudaStream_t s) {
    dim3 grid(ngen), b(W / 2);
    switch (kind) {
    case -1: k_gen64x2<N, W, B, -1><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 0: k_gen64x2<N, W, B, 0><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 1: k_gen64x2<N, W, B, 1><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 2: k_gen64x2<N, W, B, 2><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 3: k_gen64x2<N, W, B, 3><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    case 4: k_gen64x2<N, W, B, 4><<<grid, b, 0, s>>>(params, pidx, states, out, n, os); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int N, int TN, int B>
static cudaError_t gen32_kind(int kind, const DevParams32 *params, const int *pidx,
                              uint32_t *states, int ngen, void *out, uint64_t n,
                              uint64_t os, cudaStream_t s, int core) {
    dim3 grid(ngen), block(TN);
    if (core == 4) return gen32xk<N, TN, B, 4>(kind, params, pidx, states, ngen, out, n, os, s);
    if (core != 1) return gen32xk<N, TN, B, 2>(kind, params, pidx, states, ngen, out, n, os, s);
    switch (kind) {
    case -1: k_gen32<N, TN, B, -1><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 0: k_gen32<N, TN, B, 0><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 1: k_gen32<N, TN, B, 1><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 2: k_gen32<N, TN, B, 2><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 3: k_gen32<N, TN, B, 3><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 4: k_gen32<N, TN, B, 4><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int N, int TN, int B>
static cudaError_t gen64_kind(int kind, const DevParams64 *params, const int *pidx,
                              uint64_t *states, int ngen, void *out, uint64_t n,
                              uint64_t os, cudaStream_t s, int core) {
    dim3 grid(ngen), block(TN);
    if (core != 1) return gen64x2<N, TN, B>(kind, params, pidx, states, ngen, out, n, os, s);
    switch (kind) {
    case -1: k_gen64<N, TN, B, -1><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 0: k_gen64<N, TN, B, 0><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 1: k_gen64<N, TN, B, 1><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 2: k_gen64<N, TN, B, 2><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 3: k_gen64<N, TN, B, 3><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    case 4: k_gen64<N, TN, B, 4><<<grid, block, 0, s>>>(params, pidx, states, out, n, os); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launchGen32(int mexp, int kind, const DevParams32 *params, const int *pidx,
                        uint32_t *states, int ngen, void *out, uint64_t n,
                        uint64_t os, cudaStream_t s, int core) {
    if (ngen <= 0 || n == 0) return cudaSuccess;
#define X(M, N, T, B) \
    if (mexp == M) return gen32_kind<N, T, B>(kind, params, pidx, states, ngen, out, n, os, s, core);
    MTGP_SHAPES32(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchGen64(int mexp, int kind, const DevParams64 *params, const int *pidx,
                        uint64_t *states, int ngen, void *out, uint64_t n,
                        uint64_t os, cudaStream_t s, int core) {
    if (ngen <= 0 || n == 0) return cudaSuccess;
#define X(M, N, T, B) \
    if (mexp == M) return gen64_kind<N, T, B>(kind, params, pidx, states, ngen, out, n, os, s, core);
    MTGP_SHAPES64(X)
#undef X
    return cudaErrorInvalidValue;
}

}  // namespace mtgp
