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

template <class Tr, class Geo>
cudaError_t launch(const typename Tr::P *params, typename Tr::W *states,
                   const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    using W = typename Tr::W;
    const size_t smem = Geo::template bytes<W>(nwords);
    auto kern = k_jump<Tr, Geo>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    if (ndesc <= 0) return cudaSuccess;
    kern<<<ndesc, Geo::NT, smem, s>>>(params, states, descs, nwords);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchJump32(int mexp, const DevParams32 *params, uint32_t *states,
                         const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    constexpr int T = kJumpThreads;
    switch (mexp) {
    case 11213: return launch<Tr32, JGeo<351, 11, T, 256, 2048>>(params, states, descs, ndesc, nwords, s);
    case 23209: return launch<Tr32, JGeo<726, 23, T, 256, 4096>>(params, states, descs, ndesc, nwords, s);
    case 44497: return launch<Tr32, JGeo<1391, 45, T, 256, 4096>>(params, states, descs, ndesc, nwords, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launchJump64(int mexp, const DevParams64 *params, uint64_t *states,
                         const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    constexpr int T = kJumpThreads;
    switch (mexp) {
    case 11213: return launch<Tr64, JGeo<176, 7, T, 128, 2048>>(params, states, descs, ndesc, nwords, s);
    case 23209: return launch<Tr64, JGeo<363, 13, T, 256, 2048>>(params, states, descs, ndesc, nwords, s);
    case 44497: return launch<Tr64, JGeo<696, 23, T, 256, 4096>>(params, states, descs, ndesc, nwords, s);
    case 110503: return launch<Tr64, JGeo<1727, 27, T, 256, 4096>>(params, states, descs, ndesc, nwords, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace mtgp
