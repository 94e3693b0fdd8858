// seed_kernels.cu -- the reference's integer seeding on the device
// (mtgp32_init_state, mtgp32-fast.c:119-137; mtgp64_init_state,
// mtgp64-fast.c:124-142), one thread per stream: every word of the window is
// filled from the parameter set's hidden word, then word 0 takes the seed
// and each later word mixes in its predecessor.  A thread's 351 (or 176)
// words form one sequential chain; streams are independent, so thousands of
// streams are seeded in one launch of a few microseconds.
#include "internal.h"

namespace mtgp {
namespace {

template <typename W> struct SeedMix;
template <> struct SeedMix<uint32_t> {
    static constexpr uint32_t mul = 1812433253u;
    static constexpr int shr = 30;
    static constexpr uint32_t bytes = 0x01010101u;
    static __device__ uint32_t top(uint32_t h) { return h; }
};
template <> struct SeedMix<uint64_t> {
    static constexpr uint64_t mul = 6364136223846793005ULL;
    static constexpr int shr = 62;
    static constexpr uint64_t bytes = 0x0101010101010101ULL;
    static __device__ uint64_t top(uint64_t h) { return h >> 32; }
};

template <typename W, class P>
__global__ void k_seed(const P *__restrict__ params, const int *__restrict__ pidx,
                       const W *__restrict__ seeds, W *__restrict__ states, int count, int size,
                       int stride) {
    using M = SeedMix<W>;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const P &p = params[pidx[i]];
    const W hidden = p.tbl[4] ^ (p.tbl[8] << 16);
    W b = M::top(hidden);
    b += b >> 16;
    b += b >> 8;
    const W fill = (b & 0xffu) * M::bytes;
    W *a = states + (size_t)i * stride;
    W prev = seeds[i];
    a[0] = prev;
    for (int k = 1; k < size; k++) {
        prev = (k == 1 ? hidden : fill) ^ (M::mul * (prev ^ (prev >> M::shr)) + (W)k);
        a[k] = prev;
    }
}

}  // namespace

cudaError_t launchSeed32(const DevParams32 *params, const int *pidx, const uint32_t *seeds,
                         uint32_t *states, int count, int size, int stride, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_seed<uint32_t, DevParams32><<<(count + 127) / 128, 128, 0, s>>>(params, pidx, seeds, states,
                                                                      count, size, stride);
    return cudaGetLastError();
}

cudaError_t launchSeed64(const DevParams64 *params, const int *pidx, const uint64_t *seeds,
                         uint64_t *states, int count, int size, int stride, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_seed<uint64_t, DevParams64><<<(count + 127) / 128, 128, 0, s>>>(params, pidx, seeds, states,
                                                                      count, size, stride);
    return cudaGetLastError();
}

}  // namespace mtgp
