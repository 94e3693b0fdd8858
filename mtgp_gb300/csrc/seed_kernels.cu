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

// Key schedules (mtgp32_init_by_array, mtgp32-fast.c:151-235, and
// init_by_str, :250-334; 64-bit twins mtgp64-fast.c:156-239 / 255-339), one
// thread per stream.  keys[koff[i] .. koff[i+1]) are stream i's key words as
// the reference adds them (array words, or string bytes as signed char); the
// window is filled like the integer seeding's, then three passes mix keys
// and positions in.  The passes read and write four positions of the
// thread's own window per step (a dependent chain); the window lives in the
// stream's state row, cached by L1.
template <typename W> struct KeyMix;
template <> struct KeyMix<uint32_t> {
    static constexpr uint32_t mul1 = 1664525u, mul2 = 1566083941u;
    static constexpr int shr = 27;
};
template <> struct KeyMix<uint64_t> {
    static constexpr uint64_t mul1 = 2173292883993ULL, mul2 = 58885565329898161ULL;
    static constexpr int shr = 59;
};

template <typename W, class P>
__global__ void k_keyed(const P *__restrict__ params, const int *__restrict__ pidx,
                        const W *__restrict__ keys, const uint64_t *__restrict__ koff,
                        W *__restrict__ states, int count, int size, int stride) {
    using M = SeedMix<W>;
    using K = KeyMix<W>;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= count) return;
    const P &p = params[pidx[s]];
    const W hidden = p.tbl[4] ^ (p.tbl[8] << 16);
    W b = M::top(hidden);
    b += b >> 16;
    b += b >> 8;
    const W fill = (b & 0xffu) * M::bytes;
    W *a = states + (size_t)s * stride;
    for (int k = 1; k < size; k++) a[k] = fill;
    a[0] = hidden;
    const int lag = size >= 623 ? 11 : size >= 68 ? 7 : size >= 39 ? 5 : 3;
    const int mid = (size - lag) / 2;
    const W *key = keys + koff[s];
    const int len = (int)(koff[s + 1] - koff[s]);
    auto f1 = [](W x) { return (W)((x ^ (x >> K::shr)) * K::mul1); };
    auto f2 = [](W x) { return (W)((x ^ (x >> K::shr)) * K::mul2); };
    const int total = (len + 1 > size ? len + 1 : size) - 1;
    W r = f1(a[0] ^ a[mid] ^ a[size - 1]);
    a[mid] += r;
    r += (W)len;
    a[(mid + lag) % size] += r;
    a[0] = r;
    // i runs 1, 2, ..., size - 1, 0, 1, ...; the other positions follow it
    int i = 1, im = (1 + mid) % size, iml = (1 + mid + lag) % size, ip = 0;
    auto next = [&]() {
        ip = i;
        i = i + 1 == size ? 0 : i + 1;
        im = im + 1 == size ? 0 : im + 1;
        iml = iml + 1 == size ? 0 : iml + 1;
    };
    for (int j = 0; j < total; j++) {
        W t = f1(a[i] ^ a[im] ^ a[ip]);
        a[im] += t;
        t += (j < len ? key[j] : (W)0) + (W)i;
        a[iml] += t;
        a[i] = t;
        next();
    }
    for (int j = 0; j < size; j++) {
        W t = f2(a[i] + a[im] + a[ip]);
        a[im] ^= t;
        t -= (W)i;
        a[iml] ^= t;
        a[i] = t;
        next();
    }
    if (a[size - 1] == 0) a[size - 1] = (W)0x4d544750u;
}

}  // namespace

cudaError_t launchKeyed32(const DevParams32 *params, const int *pidx, const uint32_t *keys,
                          const uint64_t *koff, uint32_t *states, int count, int size, int stride,
                          cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_keyed<uint32_t, DevParams32><<<(count + 63) / 64, 64, 0, s>>>(params, pidx, keys, koff,
                                                                    states, count, size, stride);
    return cudaGetLastError();
}

cudaError_t launchKeyed64(const DevParams64 *params, const int *pidx, const uint64_t *keys,
                          const uint64_t *koff, uint64_t *states, int count, int size, int stride,
                          cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_keyed<uint64_t, DevParams64><<<(count + 63) / 64, 64, 0, s>>>(params, pidx, keys, koff,
                                                                    states, count, size, stride);
    return cudaGetLastError();
}

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
