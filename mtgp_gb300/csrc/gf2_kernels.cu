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
// its 2^WIN multiples v * B (v < 2^WIN; WIN = 4 bits, 2 for polynomials too
// long for that table) in shared memory; the word A[i] of the left operand
// contributes, for each WIN-bit window w of A[i] with value v, the table row
// v shifted by 32 i + WIN w bits.  A warp takes a tile of 32 K output words
// x 32 words of A: lane l owns word l of each of K blocks of 32 output words
// and keeps one accumulator per (block, window position), so that one
// window extraction serves K table loads (consecutive words across the
// lanes: no bank conflicts) and two loads share one three-input XOR.  The
// kernel is then bound by shared-memory bandwidth (one 128-byte wavefront per
// warp-wide load).  The window shifts are applied once per tile, the bits
// that cross into the next word pass one lane up with a shuffle, and the
// tile adds its words to the result with shared-memory XOR atomics.  Table
// rows carry zero padding (32 words before, 32 K + 32 after) so that no
// lane of a visited tile needs a bounds test.  There is no carry-less
// multiply instruction; a table load stands for WIN shifted XORs.
#include "internal.h"

namespace mtgp {
namespace {

constexpr int kPowThreads = 1024;

// Output words per lane: K blocks of 32 words (one window extraction serves
// K table loads); the K x NB accumulators of a lane take 32 registers.  A
// tile covers IL words of A.
template <int WIN>
struct Comb {
    static constexpr int NB = 32 / WIN;  // windows per word
    static constexpr int K = NB == 8 ? 4 : 2;
    static constexpr int IL = 32;
    static constexpr int kPadLo = 32, kPadHi = 32 * K + 32;
};

template <int WIN>
__host__ __device__ constexpr int rowStride(int W) {
    return Comb<WIN>::kPadLo + W + 1 + Comb<WIN>::kPadHi;
}

// shared words: table (2^WIN rows), R (W), P (2W + 2), Q (W + 1), U (2W + 2)
template <int WIN>
__host__ __device__ constexpr size_t powSmemWords(int W) {
    return (size_t)(1 << WIN) * rowStride<WIN>(W) + (size_t)W + (2 * W + 2) + (W + 1) +
           (2 * W + 2);
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
        T[v * S + Comb<WIN>::kPadLo + d] = w;
    }
    __syncthreads();
}

// Out[o] ^= (A * B)[o] for o in [o_lo, o_hi); A: la words (generic
// pointer), B: lb words through its table T.  Ends with a barrier.
//
// The words of A block ib (IL words) meet the output blocks (32 words) ob
// with 0 <= 32 ob - IL ib + 31 and 32 ob - IL ib - IL + 1 <= lb: a run of
// consecutive blocks, cut into tiles of K blocks from its first (the last
// tile may reach past the run and reads the rows' zero padding).  The
// tiles' A-word pairs are dealt out to the warps in equal contiguous
// ranges, so that no warp waits for another at the closing barrier; a tile
// split between warps adds its partial sums with the same atomics.
template <int WIN>
__device__ void combMul(const uint32_t *A, int la, const uint32_t *T, int S, int lb,
                        uint32_t *Out, int o_lo, int o_hi) {
    constexpr int NB = Comb<WIN>::NB, K = Comb<WIN>::K, IL = Comb<WIN>::IL, PAIRS = IL / 2;
    constexpr int MASK = (1 << WIN) - 1, nwarps = kPowThreads / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nib = (la + IL - 1) / IL;
    const int ob_lo = (o_lo > 0 ? o_lo - 1 : 0) >> 5;  // o_lo - 1 may carry into o_lo
    const int ob_hi = (o_hi - 1) >> 5;
    // output blocks of A block b: [first(b), last(b)]
    auto first = [&](int b) {
        const int f = (IL * b) >> 5;  // 32 ob + 31 >= IL b
        return f > ob_lo ? f : ob_lo;
    };
    auto last = [&](int b) {
        const int l = (IL * b + IL - 1 + lb) >> 5;  // 32 ob <= IL b + IL - 1 + lb
        return l < ob_hi ? l : ob_hi;
    };
    auto cnt = [&](int b) {
        const int n = last(b) - first(b) + 1;
        return n > 0 ? (n + K - 1) / K : 0;
    };
    int tiles = 0;
    for (int b = 0; b < nib; b++) tiles += cnt(b);
    const int units = tiles * PAIRS;
    const int u1 = (int)(((long long)(warp + 1) * units) / nwarps);
    int u = (int)(((long long)warp * units) / nwarps);
    int ib = 0, base = 0;  // base: index of A block ib's first tile
    while (u < u1) {
        const int t = u / PAIRS, p0 = u - t * PAIRS;
        const int p1 = p0 + (u1 - u) < PAIRS ? p0 + (u1 - u) : PAIRS;
        u += p1 - p0;
        while (t >= base + cnt(ib)) {
            base += cnt(ib);
            ib++;
        }
        const int ob = first(ib) + K * (t - base);
        const int o = (ob << 5) + lane, ia = IL * ib + lane;
        const uint32_t areg = (lane < IL && ia < la) ? A[ia] : 0u;
        uint32_t acc[K][NB];
#pragma unroll
        for (int k = 0; k < K; k++)
#pragma unroll
            for (int w = 0; w < NB; w++) acc[k][w] = 0;
        // word d = o + 32 k - i of the rows, i = IL ib + il:
        // -31 <= d <= lb + 32 K + IL - 2 over a visited tile
        const uint32_t *tp = T + Comb<WIN>::kPadLo + o - IL * ib;
#pragma unroll 1
        for (int il = 2 * p0; il < 2 * p1; il += 2) {
            const uint32_t a0 = __shfl_sync(0xffffffffu, areg, il);
            const uint32_t a1 = __shfl_sync(0xffffffffu, areg, il + 1);
            if (a0 | a1) {  // the same words for the whole warp
#pragma unroll
                for (int w = 0; w < NB; w++) {
                    const uint32_t *q0 = tp - il + (int)((a0 >> (WIN * w)) & MASK) * S;
                    const uint32_t *q1 = tp - il - 1 + (int)((a1 >> (WIN * w)) & MASK) * S;
#pragma unroll
                    for (int k = 0; k < K; k++) acc[k][w] ^= q0[32 * k] ^ q1[32 * k];
                }
            }
        }
        // window shifts; bits crossing into the next word move one lane up
        // (lane 31's to lane 0 of the next block, the last block's to the
        // word after the tile)
        uint32_t carry = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            uint32_t lo = acc[k][0], hi = 0;
#pragma unroll
            for (int w = 1; w < NB; w++) {
                lo ^= acc[k][w] << (WIN * w);
                hi ^= acc[k][w] >> (32 - WIN * w);
            }
            const uint32_t up = __shfl_sync(0xffffffffu, hi, (lane + 31) & 31);
            lo ^= lane ? up : carry;
            carry = up;  // lane 0: lane 31's bits, for the next block
            const int ok = o + 32 * k;
            if (ok >= o_lo && ok < o_hi) atomicXor(&Out[ok], lo);
        }
        const int oe = o - lane + 32 * K;
        if (lane == 0 && oe >= o_lo && oe < o_hi) atomicXor(&Out[oe], carry);
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
    const int S = rowStride<WIN>(W);
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

// Table slot of X^(2^i): 256 m + 2^b for i = 8 m + b (pow_sched.h).
__device__ __forceinline__ int pow2Slot(int i) { return (i >> 3) * 256 + (1 << (i & 7)); }

// X^(2^i) for i < i0 (monomials, 2^i < D) into the zeroed tables of n sets.
__global__ void k_monomials(uint32_t *blk, size_t tw, int W, int n, int i0) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * i0) return;
    const int j = t / i0, i = t - j * i0;
    const uint64_t deg = uint64_t(1) << i;
    blk[(size_t)j * tw + (size_t)(2 + pow2Slot(i)) * W + (deg >> 5)] = 1u << (deg & 31);
}

// out[(j * 64 + i) * W ..] = the table slot X^(2^i) of set j.
__global__ void k_gather_pow2(const uint32_t *blk, size_t tw, int W, uint32_t *out) {
    const int j = blockIdx.x / 64, i = blockIdx.x % 64;
    const uint32_t *src = blk + (size_t)j * tw + (size_t)(2 + pow2Slot(i)) * W;
    uint32_t *dst = out + (size_t)blockIdx.x * W;
    for (int w = threadIdx.x; w < W; w += blockDim.x) dst[w] = src[w];
}

constexpr size_t kPowSmemMax = 200 * 1024;

}  // namespace

bool powOpsFits(int W) { return W > 0 && powSmemWords<2>(W) * 4 <= kPowSmemMax; }

cudaError_t launchMonomials(uint32_t *blk, size_t tw, int W, int n, int i0, cudaStream_t s) {
    if (n <= 0 || i0 <= 0) return cudaSuccess;
    k_monomials<<<(n * i0 + 127) / 128, 128, 0, s>>>(blk, tw, W, n, i0);
    return cudaGetLastError();
}

cudaError_t launchGatherPow2(const uint32_t *blk, size_t tw, int W, int n, uint32_t *out,
                             cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_gather_pow2<<<n * 64, 128, 0, s>>>(blk, tw, W, out);
    return cudaGetLastError();
}

cudaError_t launchPowOps(const PowOp *ops, int n, const uint32_t *scratch, int W,
                         cudaStream_t s, int window) {
    if (n <= 0) return cudaSuccess;
    if (!powOpsFits(W)) return cudaErrorInvalidValue;
    const bool wide = window != 2 && powSmemWords<4>(W) * 4 <= kPowSmemMax;
    const size_t smem = 4 * (wide ? powSmemWords<4>(W) : powSmemWords<2>(W));
    auto kern = wide ? k_powops<4> : k_powops<2>;
    static std::atomic<size_t> seen[2][16];
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) e = allowSmem(kern, smem, seen[wide]);
    if (e != cudaSuccess) return e;
    kern<<<n, kPowThreads, smem, s>>>(ops, scratch, W);
    return cudaGetLastError();
}

}  // namespace mtgp
