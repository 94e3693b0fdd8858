// bm_kernels.cu -- characteristic polynomials and Barrett constants on the
// GPU, one warp per parameter set.
//
// Berlekamp-Massey (the reference computes chi offline with NTL's
// MinPolySeq over the LSBs of 2 * mexp outputs, mtgp32-calc-poly.cpp:36-45):
// every step N takes the discrepancy d = sum_{i <= L} C_i s[N - i] and, when
// it is 1, adds x^(N - m) B to the connection polynomial C (and swaps roles
// when the length changes).  The sequence is stored reversed, bit k of R =
// s[2n - 1 - k], so the samples s[N - i], i = 0.. are the bits of R from
// 2n - 1 - N upwards: the discrepancy is the parity of C AND (R >> (2n - 1 -
// N)), each lane taking every 32nd word, reduced across the warp with one
// redux.  The 2n steps are a dependent chain, so a warp (no block barrier)
// does one sequence; many sequences run at once (with fewer sequences than
// SMs, a CTA per sequence shares each step's words among its threads).
//
// Barrett's constant mu = floor(X^(2D) / chi): with C(x) = x^D chi(1/x) (the
// connection polynomial, C_0 = 1), reversing X^(2D) = q chi + r gives
// q_rev * C = 1 mod x^(D+1), so q_rev is the power series 1 / C(x) to D + 1
// terms: inv_0 = 1, inv_k = sum_{i=1..k} C_i inv_{k-i}.  Stored reversed
// (bit D - k = inv_k), that array is mu itself, and each step is again the
// parity of a window of it against C shifted down by one.
#include "internal.h"

namespace mtgp {
namespace {

__device__ __forceinline__ uint32_t wordAt(const uint32_t *v, int nw, int w) {
    return (w >= 0 && w < nw) ? v[w] : 0u;
}

// (v >> sh) word w, v of nw words (zero outside).
__device__ __forceinline__ uint32_t shr(const uint32_t *v, int nw, int w, int sh) {
    const int q = w + (sh >> 5), b = sh & 31;
    return __funnelshift_r(wordAt(v, nw, q), wordAt(v, nw, q + 1), b);
}

// (v << sh) word w.
__device__ __forceinline__ uint32_t shl(const uint32_t *v, int nw, int w, int sh) {
    const int q = w - (sh >> 5), b = sh & 31;
    return __funnelshift_l(wordAt(v, nw, q - 1), wordAt(v, nw, q), b);
}

// Berlekamp-Massey over the LSBs of seqs[j * n2 .. (j + 1) * n2) for j <
// nseq; C[j * nw ..] = the connection polynomial (bit i = C_i), L[j] = its
// length.  Shared memory per warp: R (nr words), C, B, T (nw words each).
template <typename W>
__global__ void k_bm(const W *__restrict__ seqs, int n2, int nseq, int nw, int nr, int wpb,
                     uint32_t *__restrict__ Cout, int *__restrict__ Lout) {
    extern __shared__ __align__(16) uint32_t sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * wpb + warp;
    if (j >= nseq) return;  // whole warps leave together
    uint32_t *R = sm + (size_t)warp * (nr + 3 * nw), *C = R + nr, *B = C + nw, *T = B + nw;
    const W *s = seqs + (size_t)j * n2;
    for (int r = 0; r < nr; r++) {
        const int k = 32 * r + lane;
        const bool bit = k < n2 && (s[n2 - 1 - k] & 1u);
        const uint32_t word = __ballot_sync(0xffffffffu, bit);
        if (lane == 0) R[r] = word;
    }
    for (int w = lane; w < nw; w += 32) C[w] = B[w] = T[w] = w == 0 ? 1u : 0u;
    T[0] = 0;
    __syncwarp();
    int L = 0, m = -1;
    for (int N = 0; N < n2; N++) {
        const int base = n2 - 1 - N;
        const int lw = L / 32 + 1;
        uint32_t acc = 0;
        for (int w = lane; w < lw; w += 32) acc ^= C[w] & shr(R, nr, w, base);
        const unsigned d = __reduce_xor_sync(0xffffffffu, __popc(acc) & 1u);
        if (d) {  // the same for the whole warp
            const int sh = N - m;
            const bool grow = 2 * L <= N;
            const int nl = grow ? N + 1 - L : L;
            const int top = (nl > L ? nl : L) / 32 + 1;
            if (grow) {  // T = C + x^sh B; then B = C, C = T
                for (int w = lane; w < top && w < nw; w += 32) T[w] = C[w] ^ shl(B, nw, w, sh);
                for (int w = top + lane; w < nw; w += 32) T[w] = 0;
                uint32_t *old = B;
                B = C;
                C = T;
                T = old;
                L = nl;
                m = N;
            } else {
                for (int w = lane; w < top && w < nw; w += 32) C[w] ^= shl(B, nw, w, sh);
            }
        }
        __syncwarp();
    }
    for (int w = lane; w < nw; w += 32) Cout[(size_t)j * nw + w] = C[w];
    if (lane == 0) Lout[j] = L;
}

// mu = floor(X^(2D) / chi) for chi of degree D: chi of set j at chi + j *
// stride, mu written at mu + j * stride (nw words each, j < n sets).
// Shared memory per warp: C' (nw words, C' bit i = C_{i+1} = chi_{D-1-i})
// and Z (nw + 2 words, the reversed series = mu).
__global__ void k_barrett(const uint32_t *__restrict__ chi, int D, int n, int nw, size_t stride,
                          int wpb, uint32_t *__restrict__ mu) {
    extern __shared__ __align__(16) uint32_t sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * wpb + warp;
    if (j >= n) return;
    uint32_t *Cp = sm + (size_t)warp * (2 * nw + 2), *Z = Cp + nw;
    const uint32_t *ch = chi + (size_t)j * stride;
    // C' word w: bits i = 32 w .. 32 w + 31 are chi bits D - 1 - i, i.e. the
    // bit reversal of chi's 32 bits ending at bit D - 1 - 32 w
    for (int w = lane; w < nw; w += 32) {
        const int lo = D - 32 - 32 * w;  // lowest chi bit of the group (may be < 0)
        uint32_t g;
        if (lo >= 0) {
            g = __funnelshift_r(ch[lo >> 5], (lo >> 5) + 1 < nw ? ch[(lo >> 5) + 1] : 0u, lo & 31);
        } else if (lo > -32) {
            g = ch[0] << (-lo);  // bits below 0 are zero
        } else {
            g = 0;
        }
        Cp[w] = __brev(g);
    }
    for (int w = lane; w < nw + 2; w += 32) Z[w] = (w == (D >> 5)) ? 1u << (D & 31) : 0u;
    __syncwarp();
    for (int k = 1; k <= D; k++) {
        // inv_k = sum_{i=1..k} C_i inv_{k-i}: C' bit i-1 against Z bit D-k+i
        const int base = D - k + 1;
        const int lw = (k - 1) / 32 + 1;
        uint32_t acc = 0;
        for (int w = lane; w < lw; w += 32) acc ^= Cp[w] & shr(Z, nw + 2, w, base);
        const unsigned d = __reduce_xor_sync(0xffffffffu, __popc(acc) & 1u);
        if (d && lane == 0) Z[(D - k) >> 5] |= 1u << ((D - k) & 31);
        __syncwarp();
    }
    for (int w = lane; w < nw; w += 32) mu[(size_t)j * stride + w] = Z[w];
}

// The same two chains with one CTA (NT threads) per sequence, for when there
// are fewer sequences than SMs: each thread takes every NT-th word, warps
// reduce with redux and the CTA with one barrier per step over
// double-buffered warp partials (a step's partials are written while
// slower threads may still read the previous step's).
constexpr int kChainThreads = 256;

__device__ __forceinline__ unsigned ctaParity(unsigned p, unsigned *red, int step) {
    constexpr int NWARP = kChainThreads / 32;
    const unsigned wp = __reduce_xor_sync(0xffffffffu, p);
    unsigned *buf = red + (step & 1) * NWARP;
    if ((threadIdx.x & 31) == 0) buf[threadIdx.x >> 5] = wp;
    __syncthreads();
    unsigned d = 0;
#pragma unroll
    for (int k = 0; k < NWARP; k++) d ^= buf[k];
    return d;
}

template <typename W>
__global__ void __launch_bounds__(kChainThreads)
k_bm_cta(const W *__restrict__ seqs, int n2, int nw, int nr, uint32_t *__restrict__ Cout,
         int *__restrict__ Lout) {
    extern __shared__ __align__(16) uint32_t sm[];
    __shared__ unsigned red[2 * (kChainThreads / 32)];
    const int tid = threadIdx.x, j = blockIdx.x;
    uint32_t *R = sm, *C = R + nr, *B = C + nw, *T = B + nw;
    const W *s = seqs + (size_t)j * n2;
    for (int r = tid >> 5; r < nr; r += kChainThreads / 32) {  // one warp per word of R
        const int k = 32 * r + (tid & 31);
        const uint32_t word = __ballot_sync(0xffffffffu, k < n2 && (s[n2 - 1 - k] & 1u));
        if ((tid & 31) == 0) R[r] = word;
    }
    for (int w = tid; w < nw; w += kChainThreads) C[w] = B[w] = (w == 0 ? 1u : 0u);
    __syncthreads();
    int L = 0, m = -1;
    for (int N = 0; N < n2; N++) {
        const int base = n2 - 1 - N;
        const int lw = L / 32 + 1;
        uint32_t acc = 0;
        for (int w = tid; w < lw; w += kChainThreads) acc ^= C[w] & shr(R, nr, w, base);
        const unsigned d = ctaParity(__popc(acc) & 1u, red, N);
        if (d) {  // the same for the whole CTA
            const int sh = N - m;
            const bool grow = 2 * L <= N;
            const int nl = grow ? N + 1 - L : L;
            const int top = (nl > L ? nl : L) / 32 + 1;
            if (grow) {
                for (int w = tid; w < nw; w += kChainThreads)
                    T[w] = w < top ? C[w] ^ shl(B, nw, w, sh) : 0u;
                uint32_t *old = B;
                B = C;
                C = T;
                T = old;
                L = nl;
                m = N;
            } else {
                for (int w = tid; w < top && w < nw; w += kChainThreads) C[w] ^= shl(B, nw, w, sh);
            }
        }
        // the next step's barrier (in ctaParity) orders these writes before
        // any thread reads another's words
    }
    __syncthreads();
    for (int w = tid; w < nw; w += kChainThreads) Cout[(size_t)j * nw + w] = C[w];
    if (tid == 0) Lout[j] = L;
}

__global__ void __launch_bounds__(kChainThreads)
k_barrett_cta(const uint32_t *__restrict__ chi, int D, int nw, size_t stride,
              uint32_t *__restrict__ mu) {
    extern __shared__ __align__(16) uint32_t sm[];
    __shared__ unsigned red[2 * (kChainThreads / 32)];
    const int tid = threadIdx.x, j = blockIdx.x;
    uint32_t *Cp = sm, *Z = Cp + nw;
    const uint32_t *ch = chi + (size_t)j * stride;
    for (int w = tid; w < nw; w += kChainThreads) {
        const int lo = D - 32 - 32 * w;
        uint32_t g;
        if (lo >= 0) {
            g = __funnelshift_r(ch[lo >> 5], (lo >> 5) + 1 < nw ? ch[(lo >> 5) + 1] : 0u, lo & 31);
        } else if (lo > -32) {
            g = ch[0] << (-lo);
        } else {
            g = 0;
        }
        Cp[w] = __brev(g);
    }
    for (int w = tid; w < nw + 2; w += kChainThreads)
        Z[w] = (w == (D >> 5)) ? 1u << (D & 31) : 0u;
    __syncthreads();
    for (int k = 1; k <= D; k++) {
        const int base = D - k + 1;
        const int lw = (k - 1) / 32 + 1;
        uint32_t acc = 0;
        for (int w = tid; w < lw; w += kChainThreads) acc ^= Cp[w] & shr(Z, nw + 2, w, base);
        const unsigned d = ctaParity(__popc(acc) & 1u, red, k);
        if (d && tid == 0) Z[(D - k) >> 5] |= 1u << ((D - k) & 31);
        // the new bit sits in the next window's lowest word, which another
        // thread reads when the window crosses a word boundary
        __syncthreads();
    }
    __syncthreads();
    for (int w = tid; w < nw; w += kChainThreads) mu[(size_t)j * stride + w] = Z[w];
}

int smCount() {
    static int sms = 0;
    if (!sms) {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            sms = v;
        else
            return 152;
    }
    return sms;
}

int warpsPerBlock(size_t per_warp_bytes) {
    int w = (int)((200 * 1024) / (per_warp_bytes ? per_warp_bytes : 1));
    return w < 1 ? 1 : w > 4 ? 4 : w;
}

template <typename W>
cudaError_t bmLaunch(const W *seqs, int n2, int nseq, int nw, uint32_t *C, int *L,
                     cudaStream_t s) {
    if (nseq <= 0) return cudaSuccess;
    const int nr = (n2 + 31) / 32 + 2;
    const size_t per = sizeof(uint32_t) * ((size_t)nr + 3 * (size_t)nw);
    if (per > 200 * 1024) return cudaErrorInvalidValue;
    if (nseq < smCount()) {  // few sequences: a CTA each
        cudaError_t e = cudaSuccess;
        if (per > 48 * 1024)
            e = cudaFuncSetAttribute(k_bm_cta<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)per);
        if (e != cudaSuccess) return e;
        k_bm_cta<W><<<nseq, kChainThreads, per, s>>>(seqs, n2, nw, nr, C, L);
        return cudaGetLastError();
    }
    const int wpb = warpsPerBlock(per);
    const size_t smem = per * wpb;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_bm<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_bm<W><<<(nseq + wpb - 1) / wpb, 32 * wpb, smem, s>>>(seqs, n2, nseq, nw, nr, wpb, C, L);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchBM32(const uint32_t *seqs, int n2, int nseq, int nw, uint32_t *C, int *L,
                       cudaStream_t s) {
    return bmLaunch<uint32_t>(seqs, n2, nseq, nw, C, L, s);
}

cudaError_t launchBM64(const uint64_t *seqs, int n2, int nseq, int nw, uint32_t *C, int *L,
                       cudaStream_t s) {
    return bmLaunch<uint64_t>(seqs, n2, nseq, nw, C, L, s);
}

cudaError_t launchBarrett(const uint32_t *chi, int D, int n, int nw, size_t stride, uint32_t *mu,
                          cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const size_t per = sizeof(uint32_t) * (2 * (size_t)nw + 2);
    if (per > 200 * 1024) return cudaErrorInvalidValue;
    if (n < smCount()) {  // few sets: a CTA each
        cudaError_t e = cudaSuccess;
        if (per > 48 * 1024)
            e = cudaFuncSetAttribute(k_barrett_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)per);
        if (e != cudaSuccess) return e;
        k_barrett_cta<<<n, kChainThreads, per, s>>>(chi, D, nw, stride, mu);
        return cudaGetLastError();
    }
    const int wpb = warpsPerBlock(per);
    const size_t smem = per * wpb;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_barrett, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_barrett<<<(n + wpb - 1) / wpb, 32 * wpb, smem, s>>>(chi, D, n, nw, stride, wpb, mu);
    return cudaGetLastError();
}

}  // namespace mtgp
