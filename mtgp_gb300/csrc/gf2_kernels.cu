// gf2_kernels.cu -- jump polynomials X^e mod chi computed on the GPU.
//
// The host's GF(2)[x] code (gf2.cpp) needs up to a few milliseconds for a
// new exponent (one product per set bit); requests at arbitrary offsets at a
// high rate need many of them at once.  Here one CTA computes one X^e mod
// chi, and many run in parallel:
//   - polynomials are arrays of 32-bit words in shared memory, bit i of the
//     array = coefficient of X^i;
//   - a product C = A * B is word-parallel: each thread owns output words;
//     all threads walk the words of A in step and, for each set bit j of a
//     word A[i] (the same for the whole CTA, so the loop is uniform), XOR
//     B shifted by 32 i + j into their outputs -- one funnel shift and one
//     XOR per set bit and output word (there is no carry-less multiply
//     instruction to emulate);
//   - reduction mod chi (degree D) is Barrett's: with mu = floor(X^(2D) /
//     chi), q = ((P >> D) * mu) >> D and P mod chi = (P - q * chi) mod X^D,
//     exact over GF(2) for deg P < 2D;
//   - X^e is the product of the cached X^(2^i) over the set bits of e.
// Results equal the host's (checked bit for bit by the tests).
#include "internal.h"

namespace mtgp {
namespace {

constexpr int kPolyThreads = 256;

// C[o] for o in [o_lo, o_hi) of A (la words) * B (lb words); every thread
// of the CTA calls it; ends with a barrier.
__device__ void pmul(const uint32_t *A, int la, const uint32_t *B, int lb, uint32_t *C,
                     int o_lo, int o_hi) {
    constexpr int K = 3;  // outputs per thread per pass (768: 2 x 351 words in one)
    for (int base = o_lo; base < o_hi; base += K * kPolyThreads) {
        uint32_t acc[K];
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] = 0;
        for (int i = 0; i < la; i++) {
            const uint32_t a = A[i];
            if (!a) continue;
            uint32_t hi[K], lo[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                const int o = base + (int)threadIdx.x + k * kPolyThreads;
                const int bh = o - i, bl = o - i - 1;  // words of B that land on o
                hi[k] = (o < o_hi && bh >= 0 && bh < lb) ? B[bh] : 0u;
                lo[k] = (o < o_hi && bl >= 0 && bl < lb) ? B[bl] : 0u;
            }
            for (uint32_t m = a; m; m &= m - 1) {
                const int j = __ffs(m) - 1;
#pragma unroll
                for (int k = 0; k < K; k++) acc[k] ^= __funnelshift_l(lo[k], hi[k], j);
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int o = base + (int)threadIdx.x + k * kPolyThreads;
            if (o < o_hi) C[o] = acc[k];
        }
    }
    __syncthreads();
}

// dst[0..n) = src >> sh bits (src holds at least n + sh/32 + 1 words).
__device__ void pshr(const uint32_t *src, int sh, uint32_t *dst, int n) {
    const int ws = sh >> 5, bs = sh & 31;
    for (int w = threadIdx.x; w < n; w += kPolyThreads)
        dst[w] = __funnelshift_r(src[w + ws], src[w + ws + 1], bs);
    __syncthreads();
}

// R = A * B mod chi (A, B, R: W words; chi and mu: W words each, degree D).
// Scratch: P (2W + 2 words), Q (W + 1), T (2W + 2).
__device__ void pmulmod(const uint32_t *A, const uint32_t *B, const uint32_t *chi,
                        const uint32_t *mu, int D, int W, uint32_t *R, uint32_t *P,
                        uint32_t *Q, uint32_t *T) {
    for (int w = threadIdx.x; w < 2 * W + 2; w += kPolyThreads) P[w] = 0;
    __syncthreads();
    pmul(A, W, B, W, P, 0, 2 * W);                 // deg P <= 2D - 2
    pshr(P, D, Q, W);                              // Q = P >> D
    for (int w = threadIdx.x; w < 2 * W + 2; w += kPolyThreads) T[w] = 0;
    __syncthreads();
    pmul(Q, W, mu, W, T, D >> 5, 2 * W);           // the words of Q * mu at and above X^D
    pshr(T, D, Q, W);                              // q = (Q * mu) >> D
    pmul(Q, W, chi, W, T, 0, W);                   // the low W words of q * chi
    const int top = D & 31;                        // bits of the last word below X^D
    for (int w = threadIdx.x; w < W; w += kPolyThreads) {
        uint32_t v = P[w] ^ T[w];
        if (w == W - 1 && top) v &= (1u << top) - 1u;
        R[w] = v;
    }
    __syncthreads();
}

// One CTA per exponent: out[job] = prod over set bits i of steps[job] of
// p2[i] (= X^(2^i) mod chi), reduced mod chi.
__global__ void __launch_bounds__(kPolyThreads)
k_powx(const uint32_t *__restrict__ chi, const uint32_t *__restrict__ mu,
       const uint32_t *__restrict__ p2, int D, int W, const uint64_t *__restrict__ steps,
       uint32_t *__restrict__ out) {
    extern __shared__ __align__(16) uint32_t sm[];
    uint32_t *r = sm, *b = r + W, *c = b + W, *m = c + W, *P = m + W, *Q = P + 2 * W + 2,
             *T = Q + W + 1;
    const uint64_t e = steps[blockIdx.x];
    for (int w = threadIdx.x; w < W; w += kPolyThreads) {
        c[w] = chi[w];
        m[w] = mu[w];
        r[w] = w == 0 ? 1u : 0u;  // X^0
    }
    __syncthreads();
    bool first = true;
    for (int i = 0; i < 64; i++) {
        if (!((e >> i) & 1u)) continue;
        const uint32_t *pi = p2 + (size_t)i * W;
        if (first) {
            for (int w = threadIdx.x; w < W; w += kPolyThreads) r[w] = pi[w];
            __syncthreads();
            first = false;
            continue;
        }
        for (int w = threadIdx.x; w < W; w += kPolyThreads) b[w] = pi[w];
        __syncthreads();
        pmulmod(r, b, c, m, D, W, r, P, Q, T);
    }
    uint32_t *o = out + (size_t)blockIdx.x * W;
    for (int w = threadIdx.x; w < W; w += kPolyThreads) o[w] = r[w];
}

}  // namespace

// r, b, chi, mu (W words each), P (2W + 2), Q (W + 1), T (2W + 2)
size_t powxSharedBytes(int W) { return sizeof(uint32_t) * (size_t)(9 * W + 5); }

cudaError_t launchPowX(const uint32_t *chi, const uint32_t *mu, const uint32_t *p2, int D, int W,
                       const uint64_t *steps, int n, uint32_t *out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (W != D / 32 + 1) return cudaErrorInvalidValue;
    const size_t smem = powxSharedBytes(W);
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_powx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_powx<<<n, kPolyThreads, smem, s>>>(chi, mu, p2, D, W, steps, out);
    return cudaGetLastError();
}

}  // namespace mtgp
