// mtgp_device64x2.cuh -- 64-bit generation core, two adjacent words per
// thread.
//
// The 64-bit recursion and tempering of mtgp_device.cuh (sub64:
// mtgp64-fast.h:148-169, 202-249, 262-356) with the layout of the 32-bit
// K-word core (mtgp_device4.cuh): thread t of a sub-step produces the two
// consecutive sequence words N+base+2t and N+base+2t+1.  Their inputs
// overlap, so a thread loads six words (x1/x2 of both: three, the tempering
// word and y of both: three) for two outputs instead of eight, and the two
// outputs leave as one 128-bit store.  W/2 threads run one generator (64 for
// MEXP 11213).
//
// Shared layout: two planes, sequence position j in plane j & 1 at offset
// j >> 1, so the loads of a warp are consecutive 64-bit words of one plane.
// A warp's 64-bit access is two 128-byte wavefronts (half-warps); the
// planes are staggered by 8 words (64 bytes, half the banks), so that a
// half-warp copying 16 consecutive window positions (8 per plane) uses
// every bank once.
//
// Output alignment: the 128-bit store needs the item's output and the
// thread's first word 16-byte aligned.  If the item's output is only
// 8-byte aligned, its first word is produced by a one-warp pre-step and the
// rest of the item runs with the sequence phase shifted by one.
#pragma once
#include "mtgp_device4.cuh"

namespace mtgp {

template <int N, int W, int B>
struct Geo64x2 {
    static constexpr int K = 2;
    static constexpr int T = W / K;              // threads per generator
    static constexpr int PW = B / K + 8;         // words per plane (staggered)
    static constexpr int BUF = K * PW;           // 64-bit words of the buffer
    static constexpr int STEP = W / K;           // plane offset advance per sub-step
    static constexpr int S = (B - N - (K - 1)) / W;  // sub-steps per segment
    static_assert(W % (32 * K) == 0 && B % K == 0, "bad geometry");
    static_assert(S >= 2 && S * W >= N + K - 1 && S * W + N + K - 1 <= B,
                  "bad segment geometry");
};

template <int KIND> struct VecOut64 {
    using V = typename std::conditional<KIND == 0, ulonglong2, double2>::type;
    template <typename T>
    __device__ static V make(const T *v) { return V{v[0], v[1]}; }
};

// mtgp64_do_recursion (mtgp64-fast.h:148-169) from x1, x2, y; the table word
// is looked up with the low half of the result.
__device__ __forceinline__ uint64_t rec64(uint64_t x1, uint64_t x2, uint64_t y,
                                          const Lane64 &L, uint32_t mul1) {
    const uint64_t x = (x1 & L.mask) ^ x2;
    uint32_t xh = (uint32_t)(x >> 32), xl = (uint32_t)x;
    uint32_t yh = (uint32_t)(y >> 32), yl = (uint32_t)y;
    xh ^= xh * mul1;
    xl ^= xl * mul1;
    yh = xl ^ (yh >> L.sh2);
    yl = xh ^ (yl >> L.sh2);
    return (((uint64_t)yh << 32) | yl) ^ lut64(L.tbl_lo, L.tbl_hi, yl);
}

template <int N, int W, int B, int KIND>
struct Core64x2 {
    using G = Geo64x2<N, W, B>;
    static constexpr int K = 2;
    using OT = typename Out64<(KIND < 0 ? 0 : KIND)>::T;
    using VO = VecOut64<(KIND < 0 ? 0 : KIND)>;

    __device__ static __forceinline__ int at(int j) { return (j & 1) * G::PW + (j >> 1); }

    // Copy the window at positions [src, src+N) to [dst, dst+N); all threads;
    // ends with a barrier.
    __device__ static __forceinline__ void move(uint64_t *buf, int src, int dst) {
        constexpr int PER = (N + G::T - 1) / G::T;
        uint64_t v[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int k = threadIdx.x + i * G::T;
            if (k < N) v[i] = buf[at(src + k)];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < PER; i++) {
            int k = threadIdx.x + i * G::T;
            if (k < N) buf[at(dst + k)] = v[i];
        }
        __syncthreads();
    }

    struct Idx {
        int x[K + 1], y[K + 1], w[K];
    };

    __device__ static __forceinline__ Idx indices(int phase, int pos) {
        Idx I;
        const int t = threadIdx.x;
#pragma unroll
        for (int c = 0; c <= K; c++) {
            I.x[c] = at(phase + c) + t;
            I.y[c] = at(phase + pos - 1 + c) + t;
        }
#pragma unroll
        for (int c = 0; c < K; c++) I.w[c] = at(N + phase + c) + t;
        return I;
    }

    // Sub-step k of a segment: two words per thread.  GUARD: the last,
    // partial sub-step (valid = words of this thread inside n).
    template <bool GUARD>
    __device__ static __forceinline__ void sub(uint64_t *buf, const Idx &I, int k,
                                               const Lane64 &L, uint32_t mul1, uint32_t olo,
                                               uint32_t ohi, OT *o, int valid) {
        const int d = k * G::STEP;
        uint64_t xs[K + 1], ys[K + 1];
#pragma unroll
        for (int c = 0; c <= K; c++) xs[c] = buf[I.x[c] + d];
#pragma unroll
        for (int c = 0; c <= K; c++) ys[c] = buf[I.y[c] + d];
        uint64_t r[K], ov[K];
#pragma unroll
        for (int c = 0; c < K; c++) {
            r[c] = rec64(xs[c], xs[c + 1], ys[c + 1], L, mul1);
            if constexpr (KIND >= 0) ov[c] = lut64(olo, ohi, fold((uint32_t)ys[c]));
        }
#pragma unroll
        for (int c = 0; c < K; c++) buf[I.w[c] + d] = r[c];
        if constexpr (KIND >= 0) {
            OT v[K];
#pragma unroll
            for (int c = 0; c < K; c++) v[c] = Out64<KIND>::conv(r[c], ov[c]);
            if (!GUARD || valid >= K) {
                *reinterpret_cast<typename VO::V *>(o) = VO::make(v);
            } else if (valid > 0) {
                o[0] = v[0];
            }
        }
        __syncthreads();
    }

    // Advance by n steps, writing n outputs at `out` (8-byte aligned).  On
    // entry and exit the window is at positions [0, N).
    __device__ static void run(uint64_t *buf, const Lane64 &L, uint32_t olo, uint32_t ohi,
                               uint64_t n, OT *out) {
        if (n == 0) return;
        const int t = threadIdx.x;
        const uint32_t mul1 = 1u << L.sh1;
        int phase = 0;
        if constexpr (KIND >= 0) {
            phase = (int)((reinterpret_cast<uintptr_t>(out) >> 3) & 1);
            if ((uint64_t)phase > n) phase = (int)n;
        }
        if (phase > 0) {
            // position N depends only on the window; one warp computes it
            // (the table shuffles need every lane), lane 0 keeps it
            if (t < 32) {
                const uint64_t x1 = buf[at(0)], x2 = buf[at(1)], y = buf[at(L.pos)];
                const uint64_t tt = buf[at(L.pos - 1)];
                const uint64_t r = rec64(x1, x2, y, L, mul1);
                uint64_t ov = 0;
                if constexpr (KIND >= 0) ov = lut64(olo, ohi, fold((uint32_t)tt));
                if (t == 0) {
                    buf[at(N)] = r;
                    if constexpr (KIND >= 0) out[0] = Out64<(KIND < 0 ? 0 : KIND)>::conv(r, ov);
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
                sub<false>(buf, I, k, L, mul1, olo, ohi, o + k * W, K);
            move(buf, phase + (int)SEG, phase);
            n -= SEG;
            if constexpr (KIND >= 0) o += SEG;
        }
        const int rem = (int)n;
        if (rem > 0) {
            const int subs = (rem + W - 1) / W;
            for (int k = 0; k < subs; k++)
                sub<true>(buf, I, k, L, mul1, olo, ohi, o + k * W, rem - k * W - K * t);
        }
        if (phase + rem != 0) move(buf, phase + rem, 0);
    }
};

}  // namespace mtgp
