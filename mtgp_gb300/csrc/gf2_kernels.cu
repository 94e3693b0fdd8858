// gf2_kernels.cu -- products of GF(2)[x] polynomials mod chi on the GPU, the
// steps of the jump-polynomial schedules of pow_sched.h.
//
// A polynomial is an array of 32-bit words, bit i = coefficient of X^i.
// One CTA (32 warps) computes one step: R = src0; R = src_k * R mod chi for
// each further source.  One product mod chi is three polynomial products:
//   P = A * B;  q = ((P >> D) * mu) >> D;  R = (P ^ q * chi) mod X^D
// (Barrett's reduction with mu = floor(X^(2D) / chi), exact over GF(2) for
// deg P < 2D), the second only for the words at and above X^D, the third
// only below X^W.
//
// Products use the comb method.  The right operand B becomes a table of
// its 2^WIN multiples v * B (v < 2^WIN, WIN = 4 bits) in shared memory; the
// word A[i] of the left operand contributes, for each WIN-bit window w of
// A[i] with value v, the table row v shifted by 32 i + WIN w bits.  A warp
// takes a tile of 32 output words x 32 words of A: lane l owns output word
// o = 32 ob + l and keeps one accumulator per window position, so that each
// (A word, window) costs one table load (consecutive words across the
// lanes: no bank conflicts) and one XOR; the window shifts are applied once
// per tile, the bits that cross into word o + 1 pass to the next lane with a
// shuffle, and the tile adds its words to the result with shared-memory
// XOR atomics.  Tiles that touch no table word are never visited: a tile
// (ob, ib) contributes only if 0 <= ob - ib <= (lb + 31) / 32.  Table rows
// carry 32 zero words before and 64 after so that a tile's lanes never need
// a bounds test.  There is no carry-less multiply instruction; a table load
// stands for WIN shifted XORs.
#include "internal.h"

namespace mtgp {
namespace {

constexpr int kPowThreads = 1024;
constexpr int kPadLo = 32, kPadHi = 64;

__host__ __device__ constexpr int rowStride(int W) { return kPadLo + W + 1 + kPadHi; }

// shared words: table (2^WIN rows), R (W), P (2W + 2), Q (W + 1), U (2W + 2)
__host__ __device__ constexpr size_t powSmemWords(int win, int W) {
    return (size_t)(1 << win) * rowStride(W) + (size_t)W + (2 * W + 2) + (W + 1) + (2 * W + 2);
}

// Table rows T[v * S + kPadLo + d] = word d of v * B, d <= lb (B: lb words,
// generic pointer); the padding stays zero.  Ends with a barrier.
template <int WIN>
__device__ void buildTable(const uint32_t *B, int lb, uint32_t *T, int S) {
    constexpr int R = 1 << WIN;
    const int n = lb + 1;
    for (int x = threadIdx.x; x < R * n; x += kPowThreads) {
        const int v = x / n, d = x - v * n;
        const uint32_t hi = d < lb ? B[d] : 0u, lo = d > 0 ? B[d - 1] : 0u;
        uint32_t w = 0;
#pragma unroll
        for (int b = 0; b < WIN; b++)
            if ((v >> b) & 1) w ^= __funnelshift_l(lo, hi, b);
        T[v * S + kPadLo + d] = w;
    }
    __syncthreads();
}

// Out[o] ^= (A * B)[o] for o in [o_lo, o_hi); A: la words (generic
// pointer), B: lb words through its table T.  Ends with a barrier.
template <int WIN>
__device__ void combMul(const uint32_t *A, int la, const uint32_t *T, int S, int lb,
                        uint32_t *Out, int o_lo, int o_hi) {
    constexpr int NB = 32 / WIN, MASK = (1 << WIN) - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int nwarps = kPowThreads / 32;
    const int nib = (la + 31) >> 5;
    const int dmax = (lb + 31) >> 5;  // ob - ib in [0, dmax]
    const int ob1 = (o_hi - 1) >> 5;  // o_lo - 1 may carry into o_lo
    int ob = (o_lo > 0 ? o_lo - 1 : 0) >> 5, base = 0;
    auto ibLo = [&](int b) { return b - dmax > 0 ? b - dmax : 0; };
    auto cnt = [&](int b) {
        const int hi = b < nib - 1 ? b : nib - 1, lo = ibLo(b);
        return hi >= lo ? hi - lo + 1 : 0;
    };
    for (int tt = warp;; tt += nwarps) {
        while (ob <= ob1 && tt >= base + cnt(ob)) {
            base += cnt(ob);
            ob++;
        }
        if (ob > ob1) break;
        const int ib = ibLo(ob) + (tt - base);
        const int o = (ob << 5) + lane, ia = (ib << 5) + lane;
        const uint32_t areg = ia < la ? A[ia] : 0u;
        uint32_t acc[NB];
#pragma unroll
        for (int w = 0; w < NB; w++) acc[w] = 0;
        // word d = o - i of the rows, i = 32 ib + il; |d| stays in the padding
        const uint32_t *tp = T + kPadLo + o - (ib << 5);
#pragma unroll 2
        for (int il = 0; il < 32; il++) {
            const uint32_t a = __shfl_sync(0xffffffffu, areg, il);
            if (a) {  // the same word for the whole warp
                const uint32_t *t = tp - il;
#pragma unroll
                for (int w = 0; w < NB; w++) acc[w] ^= t[(int)((a >> (WIN * w)) & MASK) * S];
            }
        }
        uint32_t lo = acc[0], hi = 0;
#pragma unroll
        for (int w = 1; w < NB; w++) {
            lo ^= acc[w] << (WIN * w);
            hi ^= acc[w] >> (32 - WIN * w);
        }
        const uint32_t carry = __shfl_up_sync(0xffffffffu, hi, 1);
        if (lane) lo ^= carry;
        if (o >= o_lo && o < o_hi) atomicXor(&Out[o], lo);
        if (lane == 31 && o + 1 >= o_lo && o + 1 < o_hi) atomicXor(&Out[o + 1], hi);
    }
    __syncthreads();
}

__device__ void zero(uint32_t *p, int n) {
    for (int w = threadIdx.x; w < n; w += kPowThreads) p[w] = 0;
}

// R = A * R mod chi (A: generic pointer; R, P, Q, U, T in shared memory).
template <int WIN>
__device__ void mulmod(const uint32_t *A, uint32_t *R, const uint32_t *chi, const uint32_t *mu,
                       int D, int W, uint32_t *T, int S, uint32_t *P, uint32_t *Q, uint32_t *U) {
    zero(P, 2 * W + 2);
    buildTable<WIN>(R, W, T, S);
    combMul<WIN>(A, W, T, S, W, P, 0, 2 * W + 1);  // P = A * R, deg <= 2D - 2
    const int ws = D >> 5, bs = D & 31;
    for (int w = threadIdx.x; w < W; w += kPowThreads)  // Q = P >> D
        Q[w] = __funnelshift_r(P[w + ws], P[w + ws + 1], bs);
    zero(U, 2 * W + 2);
    buildTable<WIN>(mu, W, T, S);
    combMul<WIN>(Q, W, T, S, W, U, ws, 2 * W + 1);  // the words of Q * mu from X^D up
    for (int w = threadIdx.x; w < W; w += kPowThreads)  // q = (Q * mu) >> D
        Q[w] = __funnelshift_r(U[w + ws], U[w + ws + 1], bs);
    buildTable<WIN>(chi, W, T, S);
    combMul<WIN>(Q, W, T, S, W, P, 0, W);  // P ^= q * chi, below X^W
    for (int w = threadIdx.x; w < W; w += kPowThreads) {
        const uint32_t v = P[w];
        R[w] = w < ws ? v : w == ws ? (bs ? v & ((1u << bs) - 1u) : 0u) : 0u;
    }
    __syncthreads();
}

template <int WIN>
__global__ void __launch_bounds__(kPowThreads, 1)
k_powops(const PowOp *__restrict__ ops, const uint32_t *__restrict__ scratch, int W) {
    extern __shared__ __align__(16) uint32_t sm[];
    const int S = rowStride(W);
    uint32_t *T = sm, *R = T + (size_t)(1 << WIN) * S, *P = R + W, *Q = P + 2 * W + 2,
             *U = Q + W + 1;
    const PowOp &op = ops[blockIdx.x];
    zero(T, (1 << WIN) * S);  // the rows' padding
    auto src = [&](int c) -> const uint32_t * {
        return c >= 0 ? op.tab + (size_t)(2 + c) * W : scratch + (size_t)(-1 - c) * W;
    };
    if (op.nsrc == 0) {
        for (int w = threadIdx.x; w < W; w += kPowThreads) R[w] = w == 0 ? 1u : 0u;
    } else {
        const uint32_t *s0 = src(op.src[0]);
        for (int w = threadIdx.x; w < W; w += kPowThreads) R[w] = s0[w];
    }
    __syncthreads();
    for (int k = 1; k < op.nsrc; k++)
        mulmod<WIN>(src(op.src[k]), R, op.tab, op.tab + W, op.D, W, T, S, P, Q, U);
    for (int w = threadIdx.x; w < W; w += kPowThreads) op.dst[w] = R[w];
}

constexpr size_t kPowSmemMax = 200 * 1024;
int g_pow_window = 0;  // 0: 4 bits where the table fits, else 2

}  // namespace

bool powOpsFits(int W) { return W > 0 && powSmemWords(2, W) * 4 <= kPowSmemMax; }

void setPowWindow(int bits) { g_pow_window = bits; }

cudaError_t launchPowOps(const PowOp *ops, int n, const uint32_t *scratch, int W,
                         cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (!powOpsFits(W)) return cudaErrorInvalidValue;
    const bool wide = g_pow_window != 2 && powSmemWords(4, W) * 4 <= kPowSmemMax;
    const size_t smem = 4 * powSmemWords(wide ? 4 : 2, W);
    auto kern = wide ? k_powops<4> : k_powops<2>;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<n, kPowThreads, smem, s>>>(ops, scratch, W);
    return cudaGetLastError();
}

}  // namespace mtgp
