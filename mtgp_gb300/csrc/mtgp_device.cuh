// mtgp_device.cuh -- device building blocks of the MTGP recursion.
//
// One generator is advanced by one CTA.  Its live state (N words) sits in a
// shared-memory ring; each sub-step TN threads compute TN new words at once:
// thread t produces sequence word w+N from words w, w+1 and w+pos of the
// ring (mtgp32-fast.h:149-183; w = base + t), and tempers it with word
// w+pos-1 (mtgp32-fast.h:192-198, 252-267).  The reference's guarantee
// N - pos > TN (mtgp32-fast.h:96-106) makes the TN words of one sub-step
// independent, so one __syncthreads per sub-step orders them.
//
// The 16-entry recursion and tempering tables are held in lane registers
// (lane l keeps entry l & 15) and looked up with one warp shuffle: shfl.idx
// uses only bits [4:0] of the source-lane operand, so the raw word indexes
// the table directly.  The sequence is bit-identical to the reference's.
#pragma once
#include <cstdint>
#include <type_traits>

#include "internal.h"

namespace mtgp {

constexpr unsigned kFull = 0xffffffffu;

// 16-entry table lookup: lane (idx & 31) holds entry (idx & 15).
__device__ __forceinline__ uint32_t lut(uint32_t lane_val, uint32_t idx) {
    return __shfl_sync(kFull, lane_val, (int)idx);
}
__device__ __forceinline__ uint64_t lut64(uint32_t lo, uint32_t hi,
                                          uint32_t idx) {
    uint32_t l = __shfl_sync(kFull, lo, (int)idx);
    uint32_t h = __shfl_sync(kFull, hi, (int)idx);
    return ((uint64_t)h << 32) | l;
}

// mtgp32_do_recursion (mtgp32-fast.h:149-159) up to the table lookup.
__device__ __forceinline__ uint32_t rec32_pre(uint32_t x1, uint32_t x2,
                                              uint32_t y, uint32_t mask,
                                              int sh1, int sh2) {
    uint32_t x = (x1 & mask) ^ x2;
    x ^= x << sh1;
    return x ^ (y >> sh2);
}
// mtgp32_temper fold (mtgp32-fast.h:192-198): only bits [3:0] are used.
__device__ __forceinline__ uint32_t fold(uint32_t t) {
    t ^= t >> 16;
    t ^= t >> 8;
    return t;
}

// Output conversion, mtgp32-fast.h:252-346.  `o` is the table entry picked
// by the tempering fold: tmp_tbl for KIND 0, flt_tmp_tbl otherwise.
template <int KIND>
struct Out32 {
    using T = typename std::conditional<KIND == 0, uint32_t, float>::type;
    __device__ __forceinline__ static T conv(uint32_t r, uint32_t o) {
        if constexpr (KIND == MTGP_KIND_UINT) {
            return r ^ o;
        } else if constexpr (KIND == MTGP_KIND_CLOSE1_OPEN2) {
            return __uint_as_float((r >> 9) ^ o);
        } else if constexpr (KIND == MTGP_KIND_CLOSE_OPEN) {
            return __fsub_rn(__uint_as_float((r >> 9) ^ o), 1.0f);
        } else if constexpr (KIND == MTGP_KIND_OPEN_CLOSE) {
            return __fsub_rn(2.0f, __uint_as_float((r >> 9) ^ o));
        } else {
            return __fsub_rn(__uint_as_float(((r >> 9) ^ o) | 1u), 1.0f);
        }
    }
};

// mtgp64-fast.h:262-356.  Note open_open ORs the 1 in BEFORE the XOR with
// the table (mtgp64-fast.h:238-249), unlike the 32-bit generator.
template <int KIND>
struct Out64 {
    using T = typename std::conditional<KIND == 0, uint64_t, double>::type;
    __device__ __forceinline__ static T conv(uint64_t r, uint64_t o) {
        if constexpr (KIND == MTGP_KIND_UINT) {
            return r ^ o;
        } else if constexpr (KIND == MTGP_KIND_CLOSE1_OPEN2) {
            return __longlong_as_double((long long)((r >> 12) ^ o));
        } else if constexpr (KIND == MTGP_KIND_CLOSE_OPEN) {
            return __dsub_rn(__longlong_as_double((long long)((r >> 12) ^ o)), 1.0);
        } else if constexpr (KIND == MTGP_KIND_OPEN_CLOSE) {
            return __dsub_rn(2.0, __longlong_as_double((long long)((r >> 12) ^ o)));
        } else {
            return __dsub_rn(
                __longlong_as_double((long long)(((r >> 12) | 1u) ^ o)), 1.0);
        }
    }
};

// Per-lane copies of a generator's constants: lane l holds entry l & 15 of
// the recursion table, the tempering table and the float tempering table.
struct Lane32 {
    uint32_t tbl, tmp, flt, mask;
    int pos, sh1, sh2;
    __device__ __forceinline__ void load(const DevParams32 &P, int lane) {
        tbl = P.tbl[lane & 15];
        tmp = P.tmp[lane & 15];
        flt = P.flt[lane & 15];
        mask = P.mask;
        pos = P.pos;
        sh1 = P.sh1;
        sh2 = P.sh2;
    }
    // table used by output kind k (tmp_tbl for integers, flt_tmp_tbl else)
    __device__ __forceinline__ uint32_t otab(int k) const { return k == 0 ? tmp : flt; }
};

struct Lane64 {
    uint32_t tbl_lo, tbl_hi, tmp_lo, tmp_hi, dbl_lo, dbl_hi;
    uint64_t mask;
    int pos, sh1, sh2;
    __device__ __forceinline__ void load(const DevParams64 &P, int lane) {
        tbl_lo = (uint32_t)P.tbl[lane & 15];
        tbl_hi = (uint32_t)(P.tbl[lane & 15] >> 32);
        tmp_lo = (uint32_t)P.tmp[lane & 15];
        tmp_hi = (uint32_t)(P.tmp[lane & 15] >> 32);
        dbl_lo = (uint32_t)P.dbl[lane & 15];
        dbl_hi = (uint32_t)(P.dbl[lane & 15] >> 32);
        mask = P.mask;
        pos = P.pos;
        sh1 = P.sh1;
        sh2 = P.sh2;
    }
    __device__ __forceinline__ uint32_t otab_lo(int k) const { return k == 0 ? tmp_lo : dbl_lo; }
    __device__ __forceinline__ uint32_t otab_hi(int k) const { return k == 0 ? tmp_hi : dbl_hi; }
};

// mtgp64_do_recursion (mtgp64-fast.h:148-169) without the table XOR; the
// caller XORs tbl[yl & 15] (yl = low half of the result).
__device__ __forceinline__ uint64_t rec64_pre(uint64_t x1, uint64_t x2,
                                              uint64_t y, uint64_t mask,
                                              int sh1, int sh2) {
    uint64_t x = (x1 & mask) ^ x2;
    uint32_t xh = (uint32_t)(x >> 32), xl = (uint32_t)x;
    uint32_t yh = (uint32_t)(y >> 32), yl = (uint32_t)y;
    xh ^= xh << sh1;
    xl ^= xl << sh1;
    yh = xl ^ (yh >> sh2);
    yl = xh ^ (yl >> sh2);
    return ((uint64_t)yh << 32) | yl;
}

// Generation core: advance one generator by n steps inside a CTA of TN
// threads.
//
// The state lives in a linear shared buffer of B words.  On entry and on
// exit the window (oldest word first) is at buf[0 .. N).  A segment of S
// sub-steps appends S*TN words behind it (sub-step k, thread t reads words
// kTN+t, +1, +pos-1, +pos and writes word kTN+t+N); then the newest N words
// are copied back to buf[0 .. N) ("compaction").  Inside a segment every
// shared and global address is a per-thread base plus a compile-time
// offset, so the unrolled segment does no index arithmetic at all; the
// price is copying N words every S*TN outputs (351 per 3584 for MEXP 11213).
//
// x << sh1 is computed as x * 2^sh1 so that it issues on the FMA pipe rather
// than the ALU pipe.
template <int N, int TN, int B>
struct Seg {
    static constexpr int S = (B - N - TN) / TN + 1;  // sub-steps per segment
    static_assert(S >= 2 && S * TN >= N && S * TN + N <= B, "bad segment geometry");
};

// Copy buf[src .. src+N) to buf[0 .. N) (regions may overlap); all TN
// threads; ends with a barrier.
template <typename W, int N, int TN>
__device__ __forceinline__ void compact(W *buf, uint32_t src) {
    constexpr int PER = (N + TN - 1) / TN;
    W v[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        int k = threadIdx.x + i * TN;
        if (k < N) v[i] = buf[src + k];
    }
    if (src < (uint32_t)N) __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; i++) {
        int k = threadIdx.x + i * TN;
        if (k < N) buf[k] = v[i];
    }
    __syncthreads();
}

// One sub-step for 32-bit words.  px = buf + base + t, py = px + pos.
template <int N, int TN, int KIND, bool GUARD>
__device__ __forceinline__ void sub32(uint32_t *px, const Lane32 &L, uint32_t mul1,
                                      uint32_t otab,
                                      typename Out32<(KIND < 0 ? 0 : KIND)>::T *o,
                                      bool live) {
    const uint32_t *py = px + L.pos;
    uint32_t x1 = px[0], x2 = px[1], y = py[0];
    uint32_t x = (x1 & L.mask) ^ x2;
    uint32_t yy = x ^ (x * mul1) ^ (y >> L.sh2);
    uint32_t r = yy ^ lut(L.tbl, yy);
    px[N] = r;
    if constexpr (KIND >= 0) {
        uint32_t tt = py[-1];
        uint32_t ov = lut(otab, fold(tt));
        if (!GUARD || live) *o = Out32<KIND>::conv(r, ov);
    }
    __syncthreads();
}

template <int N, int TN, int KIND, bool GUARD>
__device__ __forceinline__ void sub64(uint64_t *px, const Lane64 &L, uint32_t mul1,
                                      uint32_t olo, uint32_t ohi,
                                      typename Out64<(KIND < 0 ? 0 : KIND)>::T *o,
                                      bool live) {
    const uint64_t *py = px + L.pos;
    uint64_t x1 = px[0], x2 = px[1], y = py[0];
    uint64_t x = (x1 & L.mask) ^ x2;
    uint32_t xh = (uint32_t)(x >> 32), xl = (uint32_t)x;
    uint32_t yh = (uint32_t)(y >> 32), yl = (uint32_t)y;
    xh ^= xh * mul1;
    xl ^= xl * mul1;
    yh = xl ^ (yh >> L.sh2);
    yl = xh ^ (yl >> L.sh2);
    uint64_t r = (((uint64_t)yh << 32) | yl) ^ lut64(L.tbl_lo, L.tbl_hi, yl);
    px[N] = r;
    if constexpr (KIND >= 0) {
        uint64_t tt = py[-1];
        uint64_t ov = lut64(olo, ohi, fold((uint32_t)tt));
        if (!GUARD || live) *o = Out64<KIND>::conv(r, ov);
    }
    __syncthreads();
}

// Advance by n steps writing n outputs of KIND (KIND < 0: no output).
// otab*: lane value of the output table (Lane32::otab(KIND)).
template <int N, int TN, int B, int KIND>
__device__ __forceinline__ void run32(uint32_t *buf, const Lane32 &L, uint32_t otab,
                                      uint64_t n,
                                      typename Out32<(KIND < 0 ? 0 : KIND)>::T *out) {
    constexpr int S = Seg<N, TN, B>::S;
    const int t = threadIdx.x;
    const uint32_t mul1 = 1u << L.sh1;
    uint32_t *px = buf + t;
    auto *o = out + t;
    while (n >= (uint64_t)S * TN) {
#pragma unroll
        for (int k = 0; k < S; k++)
            sub32<N, TN, KIND, false>(px + k * TN, L, mul1, otab, o + k * TN, true);
        compact<uint32_t, N, TN>(buf, S * TN);
        n -= (uint64_t)S * TN;
        if constexpr (KIND >= 0) o += S * TN;
    }
    const int rem = (int)n;  // < S*TN
    if (rem == 0) return;
    const int subs = (rem + TN - 1) / TN;
    for (int k = 0; k < subs; k++)
        sub32<N, TN, KIND, true>(px + k * TN, L, mul1, otab, o + k * TN, k * TN + t < rem);
    compact<uint32_t, N, TN>(buf, (uint32_t)rem);
}

template <int N, int TN, int B, int KIND>
__device__ __forceinline__ void run64(uint64_t *buf, const Lane64 &L, uint32_t olo,
                                      uint32_t ohi, uint64_t n,
                                      typename Out64<(KIND < 0 ? 0 : KIND)>::T *out) {
    constexpr int S = Seg<N, TN, B>::S;
    const int t = threadIdx.x;
    const uint32_t mul1 = 1u << L.sh1;
    uint64_t *px = buf + t;
    auto *o = out + t;
    while (n >= (uint64_t)S * TN) {
#pragma unroll
        for (int k = 0; k < S; k++)
            sub64<N, TN, KIND, false>(px + k * TN, L, mul1, olo, ohi, o + k * TN, true);
        compact<uint64_t, N, TN>(buf, S * TN);
        n -= (uint64_t)S * TN;
        if constexpr (KIND >= 0) o += S * TN;
    }
    const int rem = (int)n;
    if (rem == 0) return;
    const int subs = (rem + TN - 1) / TN;
    for (int k = 0; k < subs; k++)
        sub64<N, TN, KIND, true>(px + k * TN, L, mul1, olo, ohi, o + k * TN, k * TN + t < rem);
    compact<uint64_t, N, TN>(buf, (uint32_t)rem);
}

}  // namespace mtgp
