// jump_kernels.cu -- GF(2) jump-ahead of generator states on the GPU.
//
// The reference jumps a state by a polynomial p(X) = sum c_i X^i
// (mtgp32-fast-jump.c:51-79): it walks the coefficients, XOR-accumulating
// the whole state after i steps whenever c_i = 1.  With seq = the live
// window followed by the raw recursion words, the state after i steps is
// seq[i .. i+N), so the jumped window is the correlation
//
//     J[l] = XOR_{i : c_i = 1} seq[i + l],      l = 0 .. N-1,
//
// bit-identical to the reference's result (word 0 included).  This kernel
// computes it in one CTA of 256 threads per jump:
//   - seq is produced chunk by chunk in a shared-memory ring by the normal
//     parallel recursion (up to 256 words per sub-step);
//   - the chunk's taps are split over the 8 warps; lane l of a warp owns R
//     consecutive outputs and slides an R-word register window along seq,
//     so each tap costs one shared load and R masked XORs;
//   - the warps' partial sums are combined with shared-memory atomicXor.
// A descriptor may chain several polynomials (applied in order), which is
// how substream j is reached from the table of X^(4^k * 3^162) mod chi
// (cuda-sample/mtgp32-jump-kernel.cuh:383-401 does the same one jump at a
// time, with one thread stepping the recursion).
#include "mtgp_device.cuh"

namespace mtgp {

namespace {

constexpr int kJumpThreads = 256;
constexpr int kJumpWarps = kJumpThreads / 32;

struct Tr32 {
    using W = uint32_t;
    using P = DevParams32;
    using Lane = Lane32;
    __device__ static __forceinline__ W rec(W x1, W x2, W y, const Lane &L) {
        uint32_t yy = rec32_pre(x1, x2, y, L.mask, L.sh1, L.sh2);
        return yy ^ lut(L.tbl, yy);
    }
    __device__ static __forceinline__ W andm(W v, uint32_t m) { return v & m; }
    __device__ static __forceinline__ void axor(W *p, W v) { atomicXor(p, v); }
};

struct Tr64 {
    using W = uint64_t;
    using P = DevParams64;
    using Lane = Lane64;
    __device__ static __forceinline__ W rec(W x1, W x2, W y, const Lane &L) {
        uint64_t yy = rec64_pre(x1, x2, y, L.mask, L.sh1, L.sh2);
        return yy ^ lut64(L.tbl_lo, L.tbl_hi, (uint32_t)yy);
    }
    __device__ static __forceinline__ W andm(W v, uint32_t m) {
        return v & (uint64_t)(int64_t)(int32_t)m;
    }
    __device__ static __forceinline__ void axor(W *p, W v) {
        atomicXor(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
    }
};

// Compile-time geometry of one jump kernel instance.
template <int N_, int R_, int RING_, int GW_ = kJumpThreads>
struct JGeo {
    static constexpr int N = N_;
    // generation width: words per recursion sub-step, at most the shape's
    // parallel lanes (size - pos), a multiple of 32, <= kJumpThreads
    static constexpr int GW = GW_;
    static_assert(GW % 32 == 0 && GW <= kJumpThreads, "bad generation width");
    static constexpr int R = R_;              // outputs per lane (odd: no bank conflicts)
    static_assert(R <= 64, "coefficient extraction handles up to 64 taps");
    static constexpr int G = (N + 32 * R - 1) / (32 * R);  // output groups (passes)
    static constexpr int TPW = R * ((128 + R - 1) / R);    // taps per warp per chunk
    static constexpr int C = kJumpWarps * TPW;             // taps per chunk
    static constexpr int RING = RING_;
    static constexpr int NJ = (N + 3) & ~3;
    static_assert(C + N + GW <= RING, "jump ring too small");
};

template <class G>
__host__ __device__ constexpr int polyPad() { return G::C / 32 + 4; }

template <class Tr, class Geo>
__global__ void __launch_bounds__(kJumpThreads)
k_jump(const typename Tr::P *__restrict__ params, typename Tr::W *__restrict__ states,
       const JumpDesc *__restrict__ descs, int nwords) {
    using W = typename Tr::W;
    constexpr int N = Geo::N, R = Geo::R, RING = Geo::RING;
    constexpr uint32_t M = RING - 1;
    extern __shared__ __align__(16) unsigned char smem[];
    W *ring = reinterpret_cast<W *>(smem);
    W *jin = ring + RING;          // current window
    W *jout = jin + Geo::NJ;       // accumulated jumped window
    uint32_t *poly = reinterpret_cast<uint32_t *>(jout + Geo::NJ);

    const JumpDesc &D = descs[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    typename Tr::Lane L;
    L.load(params[D.pidx], lane);
    const int taps = nwords * 32;
    const int pwords = nwords + polyPad<Geo>();

    for (int k = tid; k < N; k += kJumpThreads) jin[k] = states[D.src + k];

    for (int c = 0; c < D.nchain; c++) {
        const uint32_t *pg = D.poly[c];
        for (int k = tid; k < pwords; k += kJumpThreads) poly[k] = k < nwords ? pg[k] : 0u;
        for (int k = tid; k < N; k += kJumpThreads) jout[k] = 0;
        for (int g = 0; g < Geo::G; g++) {
            for (int k = tid; k < N; k += kJumpThreads) ring[k] = jin[k];
            __syncthreads();
            int generated = N;
            const int l0 = g * 32 * R + lane * R;
            W acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            for (int cs = 0; cs < taps; cs += Geo::C) {
                // extend seq so that it covers every tap/output of this chunk
                while (generated < cs + Geo::C + N) {
                    if (tid < Geo::GW) {  // whole warps: the table shuffle needs all lanes
                        uint32_t w = (uint32_t)(generated + tid);
                        W x1 = ring[(w - N) & M];
                        W x2 = ring[(w - N + 1) & M];
                        W y = ring[(w - N + L.pos) & M];
                        ring[w & M] = Tr::rec(x1, x2, y, L);
                    }
                    __syncthreads();
                    generated += Geo::GW;
                }
                // this warp's taps: [i0, i0 + TPW)
                const int i0 = cs + warp * Geo::TPW;
                W win[R];
#pragma unroll
                for (int r = 0; r < R; r++) win[r] = ring[(uint32_t)(i0 + l0 + r) & M];
                for (int jb = 0; jb < Geo::TPW; jb += R) {
                    const int p = i0 + jb;
                    // coefficient bits of taps p .. p+R-1 (R <= 64)
                    const uint32_t bits_lo =
                        __funnelshift_r(poly[p >> 5], poly[(p >> 5) + 1], p & 31);
                    const uint32_t bits_hi =
                        R > 32 ? __funnelshift_r(poly[(p >> 5) + 1], poly[(p >> 5) + 2], p & 31)
                               : 0u;
#pragma unroll
                    for (int j = 0; j < R; j++) {
                        const uint32_t bj = j < 32 ? bits_lo : bits_hi;
                        const uint32_t m =
                            (uint32_t)((int32_t)(bj << (31 - (j & 31))) >> 31);
#pragma unroll
                        for (int r = 0; r < R; r++) acc[r] ^= Tr::andm(win[(j + r) % R], m);
                        win[j] = ring[(uint32_t)(p + l0 + R + j) & M];
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int r = 0; r < R; r++)
                if (l0 + r < N) Tr::axor(&jout[l0 + r], acc[r]);
            __syncthreads();
        }
        for (int k = tid; k < N; k += kJumpThreads) jin[k] = jout[k];
        __syncthreads();
    }
    for (int k = tid; k < N; k += kJumpThreads) states[D.dst + k] = jin[k];
}

template <class Tr, class Geo>
cudaError_t launch(const typename Tr::P *params, typename Tr::W *states,
                   const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    using W = typename Tr::W;
    size_t smem = sizeof(W) * (Geo::RING + 2 * Geo::NJ) +
                  sizeof(uint32_t) * (size_t)(nwords + polyPad<Geo>());
    auto kern = k_jump<Tr, Geo>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    if (ndesc <= 0) return cudaSuccess;
    kern<<<ndesc, kJumpThreads, smem, s>>>(params, states, descs, nwords);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchJump32(int mexp, const DevParams32 *params, uint32_t *states,
                         const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    switch (mexp) {
    case 11213: return launch<Tr32, JGeo<351, 11, 2048>>(params, states, descs, ndesc, nwords, s);
    case 23209: return launch<Tr32, JGeo<726, 23, 4096>>(params, states, descs, ndesc, nwords, s);
    case 44497: return launch<Tr32, JGeo<1391, 45, 4096>>(params, states, descs, ndesc, nwords, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launchJump64(int mexp, const DevParams64 *params, uint64_t *states,
                         const JumpDesc *descs, int ndesc, int nwords, cudaStream_t s) {
    switch (mexp) {
    case 11213: return launch<Tr64, JGeo<176, 7, 2048, 128>>(params, states, descs, ndesc, nwords, s);
    case 23209: return launch<Tr64, JGeo<363, 13, 2048>>(params, states, descs, ndesc, nwords, s);
    case 44497: return launch<Tr64, JGeo<696, 23, 4096>>(params, states, descs, ndesc, nwords, s);
    case 110503: return launch<Tr64, JGeo<1727, 27, 4096>>(params, states, descs, ndesc, nwords, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace mtgp
