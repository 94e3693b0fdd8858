// mtgp_device4.cuh -- 32-bit generation core, K = 4 (or 2) adjacent words per
// thread.
//
// Same recursion and tempering as mtgp_device.cuh (mtgp32-fast.h:149-346),
// but thread t of a sub-step produces the K consecutive sequence words
// N+base+Kt .. +K-1.  Their inputs overlap: words base+Kt .. base+Kt+K (x1,
// x2 of all K) and base+Kt+pos-1 .. base+Kt+pos+K-1 (tempering word and y of
// all K), so a thread loads 2K+2 words for K outputs instead of 4K (10 for 4,
// 6 for 2).  The K outputs are adjacent, so they leave as one 128-bit (K = 4)
// or 64-bit (K = 2) store.  K = 4 moves the fewest shared-memory wavefronts
// per word; K = 2 runs one generator on twice the threads (a long request
// finishes sooner) for a few more.
//
// Shared layout: K planes; sequence position j lives in plane j % K at
// offset j / K, so the loads of a warp (position c + Kt for fixed c) are
// consecutive words of one plane: conflict-free.  Per item, each distinct
// (plane, offset) stream gets one per-thread index register; inside the
// unrolled segment every access is that index plus a constant.
//
// Output alignment: a vector store needs the item's output address and the
// thread's first word aligned to 4K bytes.  If the item's output is only
// 4-aligned, the first (K - a) % K words are produced by a one-warp pre-step
// and the rest of the item runs with the sequence phase shifted by that
// amount (the window then sits at positions [phase, phase + N)).
#pragma once
#include "mtgp_device.cuh"

namespace mtgp {

template <int N, int W, int B, int K = 4>
struct GeoK {
    static_assert(K == 2 || K == 4, "two or four words per thread");
    static constexpr int T = W / K;             // threads per generator
    // Words per plane.  The +32/K staggers the planes across shared-memory
    // banks: a warp's 32 consecutive window positions (window load, store
    // and compaction) fall 32/K to a plane, so the planes' bank ranges then
    // tile the 32 banks without overlap.
    static constexpr int PW = B / K + 32 / K;
    static constexpr int BUF = K * PW;          // words of the shared buffer
    static constexpr int STEP = W / K;          // plane offset advance per sub-step
    static constexpr int S = (B - N - (K - 1)) / W;  // sub-steps per segment
    static_assert(W % (32 * K) == 0 && B % K == 0, "bad geometry");
    static_assert(S >= 2 && S * W >= N + K - 1 && S * W + N + K - 1 <= B,
                  "bad segment geometry");
};
template <int N, int W, int B>
using Geo4 = GeoK<N, W, B, 4>;

// Index of sequence position j in the K-plane buffer.
template <int PW, int K = 4>
__device__ __forceinline__ int plane_at(int j) {
    return (j & (K - 1)) * PW + j / K;
}

template <int K, int KIND> struct VecOut;
template <int KIND> struct VecOut<4, KIND> {
    using V = typename std::conditional<KIND == 0, uint4, float4>::type;
    template <typename T>
    __device__ static V make(const T *v) { return V{v[0], v[1], v[2], v[3]}; }
};
template <int KIND> struct VecOut<2, KIND> {
    using V = typename std::conditional<KIND == 0, uint2, float2>::type;
    template <typename T>
    __device__ static V make(const T *v) { return V{v[0], v[1]}; }
};

template <int N, int W, int B, int KIND, int K = 4>
struct CoreK {
    using G = GeoK<N, W, B, K>;
    using OT = typename Out32<(KIND < 0 ? 0 : KIND)>::T;
    using VO = VecOut<K, (KIND < 0 ? 0 : KIND)>;

    // Copy the window at positions [src, src+N) to [dst, dst+N); all threads;
    // ends with a barrier.
    __device__ static __forceinline__ void move(uint32_t *buf, int src, int dst) {
        constexpr int PER = (N + G::T - 1) / G::T;
        uint32_t v[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int k = threadIdx.x + i * G::T;
            if (k < N) v[i] = buf[plane_at<G::PW, K>(src + k)];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int k = threadIdx.x + i * G::T;
            if (k < N) buf[plane_at<G::PW, K>(dst + k)] = v[i];
        }
        __syncthreads();
    }

    // One word at position p+N from the window, by a whole warp (lane < cnt
    // keeps its result): used for the alignment pre-step.
    __device__ static __forceinline__ uint32_t one(const uint32_t *buf, const Lane32 &L,
                                                   uint32_t mul1, int p, uint32_t *r_out) {
        uint32_t x1 = buf[plane_at<G::PW, K>(p)], x2 = buf[plane_at<G::PW, K>(p + 1)];
        uint32_t y = buf[plane_at<G::PW, K>(p + L.pos)];
        uint32_t x = (x1 & L.mask) ^ x2;
        uint32_t yy = x ^ (x * mul1) ^ (y >> L.sh2);
        uint32_t r = yy ^ lut(L.tbl, yy);
        *r_out = r;
        return buf[plane_at<G::PW, K>(p + L.pos - 1)];
    }

    struct Idx {
        int x[K + 1], y[K + 1], w[K];
    };

    // Per-thread indices for sub-step 0 of a segment whose base is `phase`.
    __device__ static __forceinline__ Idx indices(int phase, int pos) {
        Idx I;
        const int t = threadIdx.x;
#pragma unroll
        for (int c = 0; c <= K; c++) {
            I.x[c] = plane_at<G::PW, K>(phase + c) + t;
            I.y[c] = plane_at<G::PW, K>(phase + pos - 1 + c) + t;
        }
#pragma unroll
        for (int c = 0; c < K; c++) I.w[c] = plane_at<G::PW, K>(N + phase + c) + t;
        return I;
    }

    // Sub-step k of a segment: K words per thread.  GUARD: the last,
    // partial sub-step (valid = words of this thread that are inside n).
    template <bool GUARD>
    __device__ static __forceinline__ void sub(uint32_t *buf, const Idx &I, int k,
                                               const Lane32 &L, uint32_t mul1, uint32_t otab,
                                               OT *o, int valid) {
        const int d = k * G::STEP;
        uint32_t xs[K + 1], ys[K + 1];
#pragma unroll
        for (int c = 0; c <= K; c++) xs[c] = buf[I.x[c] + d];
#pragma unroll
        for (int c = 0; c <= K; c++) ys[c] = buf[I.y[c] + d];
        uint32_t r[K], ov[K];
#pragma unroll
        for (int c = 0; c < K; c++) {
            uint32_t x = (xs[c] & L.mask) ^ xs[c + 1];
            uint32_t yy = x ^ (x * mul1) ^ (ys[c + 1] >> L.sh2);
            r[c] = yy ^ lut(L.tbl, yy);
            if constexpr (KIND >= 0) ov[c] = lut(otab, fold(ys[c]));
        }
#pragma unroll
        for (int c = 0; c < K; c++) buf[I.w[c] + d] = r[c];
        if constexpr (KIND >= 0) {
            OT v[K];
#pragma unroll
            for (int c = 0; c < K; c++) v[c] = Out32<KIND>::conv(r[c], ov[c]);
            if (!GUARD || valid >= K) {
                *reinterpret_cast<typename VO::V *>(o) = VO::make(v);
            } else {
#pragma unroll
                for (int c = 0; c < K; c++)
                    if (c < valid) o[c] = v[c];
            }
        }
        __syncthreads();
    }

    // Advance by n steps, writing n outputs at `out` (4-byte aligned).  On
    // entry and exit the window is at positions [0, N).
    __device__ static void run(uint32_t *buf, const Lane32 &L, uint32_t otab, uint64_t n,
                               OT *out) {
        if (n == 0) return;
        const int t = threadIdx.x;
        const uint32_t mul1 = 1u << L.sh1;
        // alignment pre-step: words until the output is 4K-byte aligned
        int phase = 0;
        if constexpr (KIND >= 0) {
            const int a = (int)((reinterpret_cast<uintptr_t>(out) >> 2) & (K - 1));
            phase = (K - a) & (K - 1);
            if ((uint64_t)phase > n) phase = (int)n;
        }
        if (phase > 0) {
            // positions N .. N+phase-1 depend only on the window
            uint32_t r = 0, tt = 0;
            if (t < 32) tt = one(buf, L, mul1, t, &r);
            if (t < 32) {
                uint32_t ov = 0;
                if constexpr (KIND >= 0) ov = lut(otab, fold(tt));
                if (t < phase) {
                    buf[plane_at<G::PW, K>(N + t)] = r;
                    if constexpr (KIND >= 0) out[t] = Out32<(KIND < 0 ? 0 : KIND)>::conv(r, ov);
                }
            }
            __syncthreads();
            n -= phase;
            if constexpr (KIND >= 0) out += phase;
        }
        const Idx I = indices(phase, L.pos);
        OT *o = out + K * t;
        constexpr uint64_t SEG = (uint64_t)G::S * W;
        while (n >= SEG) {
#pragma unroll
            for (int k = 0; k < G::S; k++)
                sub<false>(buf, I, k, L, mul1, otab, o + k * W, K);
            move(buf, phase + (int)SEG, phase);
            n -= SEG;
            if constexpr (KIND >= 0) o += SEG;
        }
        const int rem = (int)n;
        if (rem > 0) {
            const int subs = (rem + W - 1) / W;
            for (int k = 0; k < subs; k++)
                sub<true>(buf, I, k, L, mul1, otab, o + k * W, rem - k * W - K * t);
        }
        if (phase + rem != 0) move(buf, phase + rem, 0);
    }
};
template <int N, int W, int B, int KIND>
using Core4 = CoreK<N, W, B, KIND, 4>;

}  // namespace mtgp
