// jump_kernels.cu -- jump-ahead of many windows, one CTA per descriptor.
//
// Each descriptor names a source window, a destination window and a chain
// of polynomials (jump_device.cuh).  Substream j of the reference's CUDA
// sample is reached the same way, from the table of X^(4^k * 3^162) mod chi
// (cuda-sample/mtgp32-jump-kernel.cuh:383-401), but there one thread steps
// the recursion for every coefficient; here the whole CTA does.
#include "jump_device.cuh"

namespace mtgp {

namespace {

constexpr int kJumpThreads = 256;

template <class Tr, class Geo>
__global__ void __launch_bounds__(Geo::NT)
k_jump(const typename Tr::P *__restrict__ params, typename Tr::W *__restrict__ states,
       const JumpDesc *__restrict__ descs, int nwords) {
    using W = typename Tr::W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    W *smem = reinterpret_cast<W *>(smem_raw);
    const JumpDesc &D = descs[blockIdx.x];
    typename Tr::Lane L;
    L.load(params[D.pidx], threadIdx.x & 31);
    for (int k = threadIdx.x; k < Geo::N; k += Geo::NT) smem[k] = states[D.src + k];
    jump_chain<Tr, Geo>(smem, L, D.poly, D.nchain, nwords);
    for (int k = threadIdx.x; k < Geo::N; k += Geo::NT) states[D.dst + k] = smem[k];
}

// One CTA per (jump, range of tap chunks): partial correlation XOR-ed into
// the zeroed destination window (jump_device.cuh: jump_part).
template <class Tr, class Geo>
__device__ __forceinline__ void jumpPart(const typename Tr::P *__restrict__ params,
                                         const typename Tr::W *__restrict__ states,
                                         const uint32_t *__restrict__ polys, int nwords,
                                         typename Tr::W *__restrict__ dst, int stride,
                                         const JumpPart *__restrict__ parts) {
    using W = typename Tr::W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    W *smem = reinterpret_cast<W *>(smem_raw);
    const JumpPart &D = parts[blockIdx.x];
    typename Tr::Lane L;
    L.load(params[D.pidx], threadIdx.x & 31);
    for (int k = threadIdx.x; k < Geo::N; k += Geo::NT) smem[k] = states[D.src + k];
    __syncthreads();
    jump_part<Tr, Geo>(smem, L, polys + (size_t)D.poly * nwords, nwords, D.ch0, D.ch1,
                       dst + (size_t)D.dst * stride);
}

template <class Tr, class Geo>
__global__ void __launch_bounds__(Geo::NT)
k_jump_part(const typename Tr::P *__restrict__ params, const typename Tr::W *__restrict__ states,
            const uint32_t *__restrict__ polys, int nwords, typename Tr::W *__restrict__ dst,
            int stride, const JumpPart *__restrict__ parts) {
    jumpPart<Tr, Geo>(params, states, polys, nwords, dst, stride, parts);
}

// The same with at most 48 registers, five CTAs per SM, for the 32-bit
// geometries with groups of four taps: a bench step's 184 jumps × 4 parts
// then run in one wave on 152 SMs (49 registers allowed four CTAs per SM,
// 1.2 waves).
template <class Tr, class Geo>
__global__ void __launch_bounds__(Geo::NT, 5)
k_jump_part5(const typename Tr::P *__restrict__ params, const typename Tr::W *__restrict__ states,
             const uint32_t *__restrict__ polys, int nwords, typename Tr::W *__restrict__ dst,
             int stride, const JumpPart *__restrict__ parts) {
    jumpPart<Tr, Geo>(params, states, polys, nwords, dst, stride, parts);
}

template <class Tr, class Geo, class K>
cudaError_t launchPartsWith(K kern, const typename Tr::P *params, const typename Tr::W *states,
                            const uint32_t *polys, int nwords, typename Tr::W *dst, int stride,
                            const JumpPart *parts, int nparts, cudaStream_t s) {
    using W = typename Tr::W;
    const size_t smem = Geo::template bytes<W>(nwords);
    static std::atomic<size_t> seen[16];
    cudaError_t e = allowSmem(kern, smem, seen);
    if (e != cudaSuccess) return e;
    if (nparts <= 0) return cudaSuccess;
    kern<<<nparts, Geo::NT, smem, s>>>(params, states, polys, nwords, dst, stride, parts);
    return cudaGetLastError();
}

template <class Tr, class Geo>
cudaError_t launchParts(const typename Tr::P *params, const typename Tr::W *states,
                        const uint32_t *polys, int nwords, typename Tr::W *dst, int stride,
                        const JumpPart *parts, int nparts, cudaStream_t s) {
    if constexpr (sizeof(typename Tr::W) == 4 && Geo::R <= kQuadTapsMaxR)
        return launchPartsWith<Tr, Geo>(k_jump_part5<Tr, Geo>, params, states, polys, nwords, dst,
                                        stride, parts, nparts, s);
    else
        return launchPartsWith<Tr, Geo>(k_jump_part<Tr, Geo>, params, states, polys, nwords, dst,
                                        stride, parts, nparts, s);
}

template <class Geo>
int chunksOf(int nwords) { return (nwords * 32 + Geo::C - 1) / Geo::C; }

template <class Tr, class Geo>
cudaError_t launch(const typename Tr::P *params, typename Tr::W *states,
                   const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    using W = typename Tr::W;
    const size_t smem = Geo::template bytes<W>(nwords);
    auto kern = k_jump<Tr, Geo>;
    static std::atomic<size_t> seen[16];
    cudaError_t e = allowSmem(kern, smem, seen);
    if (e != cudaSuccess) return e;
    if (ndesc <= 0) return cudaSuccess;
    kern<<<ndesc, Geo::NT, smem, s>>>(params, states, descs, nwords);
    return cudaGetLastError();
}

}  // namespace

#define MTGP_JGEO32(X)                                     \
    X(11213, (JGeo<351, 11, kJumpThreads, 256, 2048>))     \
    X(23209, (JGeo<726, 23, kJumpThreads, 256, 4096>))     \
    X(44497, (JGeo<1391, 45, kJumpThreads, 256, 4096>))
#define MTGP_JGEO64(X)                                     \
    X(11213, (JGeo<176, 7, kJumpThreads, 128, 2048>))      \
    X(23209, (JGeo<363, 13, kJumpThreads, 256, 2048>))     \
    X(44497, (JGeo<696, 23, kJumpThreads, 256, 4096>))     \
    X(110503, (JGeo<1727, 27, kJumpThreads, 256, 4096>))

template <class G> struct Unwrap;
template <class G> struct Unwrap<void(G)> { using T = G; };
#define UNWRAP(G) typename Unwrap<void G>::T

cudaError_t launchJump32(int mexp, const DevParams32 *params, uint32_t *states,
                         const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
#define X(M, G) \
    if (mexp == M) return launch<Tr32, UNWRAP(G)>(params, states, descs, ndesc, nwords, s);
    MTGP_JGEO32(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchJump64(int mexp, const DevParams64 *params, uint64_t *states,
                         const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
#define X(M, G) \
    if (mexp == M) return launch<Tr64, UNWRAP(G)>(params, states, descs, ndesc, nwords, s);
    MTGP_JGEO64(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchJumpParts32(int mexp, const DevParams32 *params, const uint32_t *states,
                              const uint32_t *polys, int nwords, uint32_t *dst, int stride,
                              const JumpPart *parts, int nparts, cudaStream_t s) {
#define X(M, G)                                                                              \
    if (mexp == M)                                                                          \
        return launchParts<Tr32, UNWRAP(G)>(params, states, polys, nwords, dst, stride, parts, \
                                            nparts, s);
    MTGP_JGEO32(X)
#undef X
    return cudaErrorInvalidValue;
}

cudaError_t launchJumpParts64(int mexp, const DevParams64 *params, const uint64_t *states,
                              const uint32_t *polys, int nwords, uint64_t *dst, int stride,
                              const JumpPart *parts, int nparts, cudaStream_t s) {
#define X(M, G)                                                                              \
    if (mexp == M)                                                                          \
        return launchParts<Tr64, UNWRAP(G)>(params, states, polys, nwords, dst, stride, parts, \
                                            nparts, s);
    MTGP_JGEO64(X)
#undef X
    return cudaErrorInvalidValue;
}

int jumpChunks32(int mexp, int nwords) {
#define X(M, G) \
    if (mexp == M) return chunksOf<UNWRAP(G)>(nwords);
    MTGP_JGEO32(X)
#undef X
    return 1;
}

int jumpChunks64(int mexp, int nwords) {
#define X(M, G) \
    if (mexp == M) return chunksOf<UNWRAP(G)>(nwords);
    MTGP_JGEO64(X)
#undef X
    return 1;
}

namespace {

// Block c: win[c] = the generator's window for c = 0, zero otherwise (the
// jump parts XOR into windows 1..).
template <typename W>
__global__ void __launch_bounds__(128)
k_chunk_windows(const W *__restrict__ gen, W *__restrict__ win, int n, int stride) {
    const size_t c = blockIdx.x;
    W *dst = win + c * (size_t)stride;
    for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = c ? W(0) : gen[k];
}

template <typename W>
cudaError_t chunkWindows(const W *gen, W *win, int n, int stride, int nwin, cudaStream_t s) {
    if (nwin <= 0 || n <= 0 || n > stride) return cudaErrorInvalidValue;
    k_chunk_windows<W><<<nwin, 128, 0, s>>>(gen, win, n, stride);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchChunkWindows32(const uint32_t *gen, uint32_t *win, int n, int stride, int nwin,
                                 cudaStream_t s) {
    return chunkWindows(gen, win, n, stride, nwin, s);
}

cudaError_t launchChunkWindows64(const uint64_t *gen, uint64_t *win, int n, int stride, int nwin,
                                 cudaStream_t s) {
    return chunkWindows(gen, win, n, stride, nwin, s);
}

}  // namespace mtgp
