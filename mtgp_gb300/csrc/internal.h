// internal.h -- declarations shared by the host (C-ABI) and kernel units.
//
// Device data layout (all in HBM):
//   DevParams32 / DevParams64  one per parameter set: pos, shifts, mask and
//                              the three 16-entry tables (recursion, temper,
//                              float temper) of mtgp32-fast.h:47-58 /
//                              mtgp64-fast.h:46-57.
//   state window               one per generator: the live state, oldest word
//                              first, `size` = mexp/w + 1 words, padded to a
//                              stride of stateStride() words (a multiple of
//                              32 words, so every window starts 128-byte
//                              aligned).  Word k of the window is the
//                              reference's array[(idx - size + 1 + k) &
//                              large_mask] (mtgp32-fast.h:165-183).
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/mtgp_gpu.h"

namespace mtgp {

struct DevParams32 {
    int pos, sh1, sh2;
    uint32_t mask;
    uint32_t tbl[16];
    uint32_t tmp[16];
    uint32_t flt[16];
};

struct DevParams64 {
    int pos, sh1, sh2, pad_;
    uint64_t mask;
    uint64_t tbl[16];
    uint64_t tmp[16];
    uint64_t dbl[16];
};

// Shape of one supported Mersenne exponent: N live words, TN parallel lanes
// (threads per generator; the reference guarantees size - pos > TN,
// mtgp32-fast.h:96-106), B = words of the generation core's shared buffer
// (at most 48 KB, so static shared memory suffices).
struct Shape {
    int mexp, n, tn, buf;
};
// Per exponent: live words N, lanes TN (threads per generator; N - pos >= TN
// for every set of the reference's tables), and the shared buffer B (words)
// of the generation core (B <= 48 KB, so static shared memory suffices).
#define MTGP_SHAPES32(X) X(11213, 351, 256, 4096) X(23209, 726, 512, 8192) X(44497, 1391, 1024, 12000)
#define MTGP_SHAPES64(X) X(11213, 176, 128, 2048) X(23209, 363, 256, 4096) X(44497, 696, 512, 4096) \
    X(110503, 1727, 512, 5760)


// Dynamic shared memory of `kern` raised to at least `smem` bytes on the
// current device; the attribute call is made once per kernel, device and
// size (servers launch jump kernels for every batch).  `seen` holds, per
// device, the largest size set so far for this kernel.
template <class K>
cudaError_t allowSmem(K kern, size_t smem, std::atomic<size_t> (&seen)[16]) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 16 && seen[dev].load(std::memory_order_acquire) >= smem)
        return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && dev >= 0 && dev < 16) {
        size_t cur = seen[dev].load(std::memory_order_relaxed);
        while (cur < smem && !seen[dev].compare_exchange_weak(cur, smem)) {
        }
    }
    return e;
}

bool shape32(int mexp, Shape *s);
bool shape64(int mexp, Shape *s);

// Every device and pinned host allocation of the library goes through
// these.  With MTGP_TEST_FAIL_ALLOC=k in the environment (read once, for
// tests of the error paths), allocation number k of the process (counted
// from 0) fails with cudaErrorMemoryAllocation without calling CUDA; unset,
// they are cudaMalloc, cudaMallocAsync and cudaHostAlloc.
cudaError_t devMallocRaw(void **p, size_t bytes);
cudaError_t devMallocAsyncRaw(void **p, size_t bytes, cudaStream_t s);
cudaError_t hostAllocRaw(void **p, size_t bytes);
template <class T>
cudaError_t devMalloc(T **p, size_t bytes) {
    return devMallocRaw(reinterpret_cast<void **>(p), bytes);
}
template <class T>
cudaError_t devMallocAsync(T **p, size_t bytes, cudaStream_t s) {
    return devMallocAsyncRaw(reinterpret_cast<void **>(p), bytes, s);
}
template <class T>
cudaError_t hostAlloc(T **p, size_t bytes) {
    return hostAllocRaw(reinterpret_cast<void **>(p), bytes);
}
__host__ __device__ constexpr int stateStride(int n) { return (n + 31) & ~31; }

void toDev(const mtgp32_params_fast_t &p, DevParams32 *d);
// Store msg as the calling thread's mtgp_gpu_last_error(); returns code.
int recordError(int code, const char *msg);

// The part of a plan's launch that reads no stream window and writes no
// output: its descriptor upload, its GPU-made jump polynomials and the
// zeroing of new pre-jumped window slots, queued on stream s.  The plan's
// next launch (or graph capture) then skips them.
int planPrepare(mtgp_gpu_plan_t *pl, void *s);
void toDev(const mtgp64_params_fast_t &p, DevParams64 *d);

// ---- generation (gen_kernels.cu) ----------------------------------------
// ngen generators, generator g uses params[pidx ? pidx[g] : g] (device
// arrays), its window at states + g*stateStride(N), and writes n values of
// `kind` at out + g*outStride elements.  kind < 0 = skip (no output).
// Integer seeding of `count` windows (size words each, `stride` apart) on
// the device: stream i from seeds[i] with parameter set pidx[i].
cudaError_t launchSeed32(const DevParams32 *params, const int *pidx, const uint32_t *seeds,
                         uint32_t *states, int count, int size, int stride, cudaStream_t s);
cudaError_t launchSeed64(const DevParams64 *params, const int *pidx, const uint64_t *seeds,
                         uint64_t *states, int count, int size, int stride, cudaStream_t s);
// Key-schedule seeding (init_by_array / init_by_str) on the device: stream
// i from the key words keys[koff[i] .. koff[i+1]).
cudaError_t launchKeyed32(const DevParams32 *params, const int *pidx, const uint32_t *keys,
                          const uint64_t *koff, uint32_t *states, int count, int size, int stride,
                          cudaStream_t s);
cudaError_t launchKeyed64(const DevParams64 *params, const int *pidx, const uint64_t *keys,
                          const uint64_t *koff, uint64_t *states, int count, int size, int stride,
                          cudaStream_t s);

// One product of a jump-polynomial schedule (pow_sched.h): dst = product
// of the nsrc sources mod chi (nsrc = 0: the polynomial 1).  tab points at
// chi | mu = floor(X^(2 D) / chi) | table slots, W words each (bit i of the
// words = coefficient of X^i); a source code >= 0 is a table slot, < 0 the
// scratch slot -1 - code.
struct PowOp {
    const uint32_t *tab;
    uint32_t *dst;
    int32_t D;  // degree of chi; W >= D / 32 + 1
    int32_t nsrc;
    int32_t src[8];
};

// The n independent products ops[0..n), one CTA each (W words per
// polynomial); smem limits: powOpsFits(W).
// Berlekamp-Massey over the LSBs of nseq sequences of n2 words (one warp
// each): connection polynomial j (bit i = C_i) at C + j * nw, length L[j].
cudaError_t launchBM32(const uint32_t *seqs, int n2, int nseq, int nw, uint32_t *C, int *L,
                       cudaStream_t s);
cudaError_t launchBM64(const uint64_t *seqs, int n2, int nseq, int nw, uint32_t *C, int *L,
                       cudaStream_t s);
// Barrett constants mu = floor(X^(2D) / chi) of n polynomials of degree D:
// chi j at chi + j * stride, mu j written at mu + j * stride (nw words).
cudaError_t launchBarrett(const uint32_t *chi, int D, int n, int nw, size_t stride, uint32_t *mu,
                          cudaStream_t s);

bool powOpsFits(int W);
// Jump tables of n sets, tw words apart: the monomial slots X^(2^i), i <
// i0; and a copy of the 64 slots X^(2^i) of each set into out (64 W words
// per set).
cudaError_t launchMonomials(uint32_t *blk, size_t tw, int W, int n, int i0, cudaStream_t s);
cudaError_t launchGatherPow2(const uint32_t *blk, size_t tw, int W, int n, uint32_t *out,
                             cudaStream_t s);
// window: bits per comb window of the products, 0 = automatic (4 where the
// table fits in shared memory, else 2), 2 or 4.
cudaError_t launchPowOps(const PowOp *ops, int n, const uint32_t *scratch, int W,
                         cudaStream_t s, int window = 0);

// core: the 32-bit generation core, 2 = two adjacent words per thread (the
// default), 4 = four, 1 = one word per thread.
cudaError_t launchGen32(int mexp, int kind, const DevParams32 *params,
                        const int *pidx, uint32_t *states, int ngen,
                        void *out, uint64_t n, uint64_t outStride,
                        cudaStream_t s, int core = 2);
// core (64-bit): 2 = two adjacent words per thread (the default, also for
// core 4), 1 = one word per thread.
cudaError_t launchGen64(int mexp, int kind, const DevParams64 *params,
                        const int *pidx, uint64_t *states, int ngen,
                        void *out, uint64_t n, uint64_t outStride,
                        cudaStream_t s, int core = 2);

// ---- jump (jump_kernels.cu) ---------------------------------------------
// One descriptor per jump.  The kernel reads the window at `src`, applies
// the polynomial (uint32-array form, nwords words), and writes the jumped
// window to `dst` (dst may equal src).  `polys` lists up to kMaxChain
// polynomials applied in order (a chain); unused entries are null.
constexpr int kMaxChain = 24;
struct JumpDesc {
    const uint32_t *poly[kMaxChain];
    int nchain;
    int pidx;          // parameter-set index
    uint64_t src;      // element offset of the source window
    uint64_t dst;      // element offset of the destination window
};
// Partial jumps: CTA b correlates the tap chunks [ch0, ch1) of one jump and
// XORs the result into its destination window (zero on entry); the parts of
// a jump together give the full jump.  jumpChunks*() = tap chunks of one
// jump.  Source windows are in `states`, polynomials in `polys` (nwords
// words each), destination windows `stride` words apart from `dst`.
struct JumpPart {
    uint64_t src;      // element offset of the source window in states
    int32_t poly;      // polynomial index
    int32_t dst;       // destination window index
    int32_t pidx;      // parameter-set index
    int16_t ch0, ch1;
};
static_assert(sizeof(JumpPart) == 24, "JumpPart is 24 bytes");
cudaError_t launchJumpParts32(int mexp, const DevParams32 *params, const uint32_t *states,
                              const uint32_t *polys, int nwords, uint32_t *dst, int stride,
                              const JumpPart *parts, int nparts, cudaStream_t s);
cudaError_t launchJumpParts64(int mexp, const DevParams64 *params, const uint64_t *states,
                              const uint32_t *polys, int nwords, uint64_t *dst, int stride,
                              const JumpPart *parts, int nparts, cudaStream_t s);
int jumpChunks32(int mexp, int nwords);
int jumpChunks64(int mexp, int nwords);
// nwin windows of `stride` words at win: window 0 = gen[0..n), the others
// zero (the destinations of jump parts).
cudaError_t launchChunkWindows32(const uint32_t *gen, uint32_t *win, int n, int stride, int nwin,
                                 cudaStream_t s);
cudaError_t launchChunkWindows64(const uint64_t *gen, uint64_t *win, int n, int stride, int nwin,
                                 cudaStream_t s);
cudaError_t launchJump32(int mexp, const DevParams32 *params, uint32_t *states,
                         const JumpDesc *descs, int ndesc, int nwords,
                         cudaStream_t s);
cudaError_t launchJump64(int mexp, const DevParams64 *params, uint64_t *states,
                         const JumpDesc *descs, int ndesc, int nwords,
                         cudaStream_t s);

}  // namespace mtgp
