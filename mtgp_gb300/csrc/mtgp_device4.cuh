// mtgp_device4.cuh -- 32-bit generation core, four adjacent words per thread.
//
// Same recursion and tempering as mtgp_device.cuh (mtgp32-fast.h:149-346),
// but thread t of a sub-step produces the four consecutive sequence words
// N+base+4t .. +3.  Their inputs overlap: words base+4t .. base+4t+4 (x1, x2
// of all four) and base+4t+pos-1 .. base+4t+pos+3 (tempering word and y of
// all four), so a thread loads 10 words for 4 outputs instead of 16.  The
// four outputs are adjacent, so they leave as one 128-bit store.
//
// Shared layout: four planes; sequence position j lives in plane j & 3 at
// offset j >> 2, so the loads of a warp (position c + 4t for fixed c) are
// consecutive words of one plane: conflict-free.  Per item, each of the 14
// distinct (plane, offset) streams gets one per-thread index register; inside
// the unrolled segment every access is that index plus a constant.
//
// Output alignment: a 128-bit store needs the item's output address and the
// thread's first word aligned to 16 bytes.  If the item's output is only
// 4-aligned, the first (4 - a) & 3 words are produced by a one-warp pre-step
// and the rest of the item runs with the sequence phase shifted by that
// amount (the window then sits at positions [phase, phase + N)).
#pragma once
#include "mtgp_device.cuh"

namespace mtgp {

template <int N, int W, int B>
struct Geo4 {
    static constexpr int T = W / 4;             // threads per generator
    // Words per plane.  The +8 staggers the planes across shared-memory
    // banks: copies that touch the four planes at the same offset (window
    // load, store and compaction) are then conflict-free.
    static constexpr int PW = B / 4 + 8;
    static constexpr int BUF = 4 * PW;          // words of the shared buffer
    static constexpr int STEP = W / 4;          // plane offset advance per sub-step
    static constexpr int S = (B - N - 3) / W;   // sub-steps per segment
    static_assert(W % 128 == 0 && B % 4 == 0, "bad geometry");
    static_assert(S >= 2 && S * W >= N + 3 && S * W + N + 3 <= B, "bad segment geometry");
};

// Index of sequence position j in the 4-plane buffer.
template <int PW>
__device__ __forceinline__ int plane_at(int j) {
    return (j & 3) * PW + (j >> 2);
}

template <int N, int W, int B, int KIND>
struct Core4 {
    using G = Geo4<N, W, B>;
    using OT = typename Out32<(KIND < 0 ? 0 : KIND)>::T;
    using O4 = typename std::conditional<KIND == 0, uint4, float4>::type;

    // Copy the window at positions [src, src+N) to [dst, dst+N); all threads;
    // ends with a barrier.
    __device__ static __forceinline__ void move(uint32_t *buf, int src, int dst) {
        constexpr int PER = (N + G::T - 1) / G::T;
        uint32_t v[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int k = threadIdx.x + i * G::T;
            if (k < N) v[i] = buf[plane_at<G::PW>(src + k)];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int k = threadIdx.x + i * G::T;
            if (k < N) buf[plane_at<G::PW>(dst + k)] = v[i];
        }
        __syncthreads();
    }

    // One word at position p+N from the window, by a whole warp (lane < cnt
    // keeps its result): used for the alignment pre-step.
    __device__ static __forceinline__ uint32_t one(const uint32_t *buf, const Lane32 &L,
                                                   uint32_t mul1, int p, uint32_t *r_out) {
        uint32_t x1 = buf[plane_at<G::PW>(p)], x2 = buf[plane_at<G::PW>(p + 1)];
        uint32_t y = buf[plane_at<G::PW>(p + L.pos)];
        uint32_t x = (x1 & L.mask) ^ x2;
        uint32_t yy = x ^ (x * mul1) ^ (y >> L.sh2);
        uint32_t r = yy ^ lut(L.tbl, yy);
        *r_out = r;
        return buf[plane_at<G::PW>(p + L.pos - 1)];
    }

    struct Idx {
        int x[5], y[5], w[4];
    };

    // Per-thread indices for sub-step 0 of a segment whose base is `phase`.
    __device__ static __forceinline__ Idx indices(int phase, int pos) {
        Idx I;
        const int t = threadIdx.x;
#pragma unroll
        for (int c = 0; c < 5; c++) {
            I.x[c] = plane_at<G::PW>(phase + c) + t;
            I.y[c] = plane_at<G::PW>(phase + pos - 1 + c) + t;
        }
#pragma unroll
        for (int c = 0; c < 4; c++) I.w[c] = plane_at<G::PW>(N + phase + c) + t;
        return I;
    }

    // Sub-step k of a segment: four words per thread.  GUARD: the last,
    // partial sub-step (valid = words of this thread that are inside n).
    template <bool GUARD>
    __device__ static __forceinline__ void sub(uint32_t *buf, const Idx &I, int k,
                                               const Lane32 &L, uint32_t mul1, uint32_t otab,
                                               OT *o, int valid) {
        const int d = k * G::STEP;
        uint32_t xs[5], ys[5];
#pragma unroll
        for (int c = 0; c < 5; c++) xs[c] = buf[I.x[c] + d];
#pragma unroll
        for (int c = 0; c < 5; c++) ys[c] = buf[I.y[c] + d];
        uint32_t r[4], ov[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint32_t x = (xs[c] & L.mask) ^ xs[c + 1];
            uint32_t yy = x ^ (x * mul1) ^ (ys[c + 1] >> L.sh2);
            r[c] = yy ^ lut(L.tbl, yy);
            if constexpr (KIND >= 0) ov[c] = lut(otab, fold(ys[c]));
        }
#pragma unroll
        for (int c = 0; c < 4; c++) buf[I.w[c] + d] = r[c];
        if constexpr (KIND >= 0) {
            OT v[4];
#pragma unroll
            for (int c = 0; c < 4; c++) v[c] = Out32<KIND>::conv(r[c], ov[c]);
            if (!GUARD || valid >= 4) {
                O4 q;
                q.x = v[0];
                q.y = v[1];
                q.z = v[2];
                q.w = v[3];
                *reinterpret_cast<O4 *>(o) = q;
            } else {
#pragma unroll
                for (int c = 0; c < 4; c++)
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
        // alignment pre-step: words until the output is 16-byte aligned
        int phase = 0;
        if constexpr (KIND >= 0) {
            const int a = (int)((reinterpret_cast<uintptr_t>(out) >> 2) & 3);
            phase = (4 - a) & 3;
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
                    buf[plane_at<G::PW>(N + t)] = r;
                    if constexpr (KIND >= 0) out[t] = Out32<(KIND < 0 ? 0 : KIND)>::conv(r, ov);
                }
            }
            __syncthreads();
            n -= phase;
            if constexpr (KIND >= 0) out += phase;
        }
        const Idx I = indices(phase, L.pos);
        OT *o = out + 4 * t;
        constexpr uint64_t SEG = (uint64_t)G::S * W;
        while (n >= SEG) {
#pragma unroll
            for (int k = 0; k < G::S; k++)
                sub<false>(buf, I, k, L, mul1, otab, o + k * W, 4);
            move(buf, phase + (int)SEG, phase);
            n -= SEG;
            if constexpr (KIND >= 0) o += SEG;
        }
        const int rem = (int)n;
        if (rem > 0) {
            const int subs = (rem + W - 1) / W;
            for (int k = 0; k < subs; k++)
                sub<true>(buf, I, k, L, mul1, otab, o + k * W, rem - k * W - 4 * t);
        }
        if (phase + rem != 0) move(buf, phase + rem, 0);
    }
};

}  // namespace mtgp
