// jump_device.cuh -- GF(2) jump-ahead of one window inside a CTA.
//
// The reference jumps a state by a polynomial p(X) = sum c_i X^i
// (mtgp32-fast-jump.c:51-79): it walks the coefficients, XOR-accumulating
// the whole state after i steps whenever c_i = 1.  With seq = the live
// window followed by the raw recursion words, the state after i steps is
// seq[i .. i+N), so the jumped window is the correlation
//
//     J[l] = XOR_{i : c_i = 1} seq[i + l],      l = 0 .. N-1,
//
// bit-identical to the reference's result (word 0 included).  One CTA of NT
// threads computes it:
//   - seq is produced chunk by chunk in a shared ring by the parallel
//     recursion (GW words per sub-step, GW <= the shape's lanes);
//   - each chunk's taps are split over the warps; lane l of a warp owns R
//     consecutive outputs and slides an R-word register window along seq,
//     so a tap costs one shared load and, when its coefficient is set, R
//     XORs; taps go in pairs (tapsR): the coefficients are the same for a
//     whole warp, so a pair is one uniform branch, a zero pair skips its
//     XORs and a pair of ones costs R three-input XORs;
//   - the warps' partial sums are combined with shared-memory atomicXor.
// A chain of polynomials is applied in order.
#pragma once
#include "mtgp_device.cuh"

namespace mtgp {

struct Tr32 {
    using W = uint32_t;
    using P = DevParams32;
    using Lane = Lane32;
    __device__ static __forceinline__ W rec(W x1, W x2, W y, const Lane &L) {
        uint32_t yy = rec32_pre(x1, x2, y, L.mask, L.sh1, L.sh2);
        return yy ^ lut(L.tbl, yy);
    }
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
    __device__ static __forceinline__ void axor(W *p, W v) {
        atomicXor(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
    }
};

// Geometry of one jump instance.
//   N    live words          R    outputs per lane (odd: conflict-free loads)
//   NT   threads of the CTA  GW   words per recursion sub-step (<= NT, <= lanes)
//   RING shared ring length (power of two), followed by MIR words that repeat
//        ring[0 .. MIR): the 2R words a tap group reads from one base are
//        then contiguous, whatever their ring position
// Shared layout, in words W: jin[NJ] | jout[NJ] | ring[RING + MIR] | poly (uint32).
template <int N_, int R_, int NT_, int GW_, int RING_>
struct JGeo {
    static constexpr int N = N_, R = R_, NT = NT_, GW = GW_, RING = RING_;
    static constexpr int NWARP = NT / 32;
    static_assert(NT % 32 == 0 && GW % 32 == 0 && GW <= NT, "bad jump widths");
    static_assert(R <= 64, "coefficient extraction handles up to 64 taps");
    static constexpr int G = (N + 32 * R - 1) / (32 * R);  // output groups (passes)
    static constexpr int TPW = R * ((128 + R - 1) / R);    // taps per warp per chunk
    static constexpr int C = NWARP * TPW;                  // taps per chunk
    static constexpr int NJ = (N + 3) & ~3;
    static constexpr int PAD = C / 32 + 4;                 // zero words after the poly
    static constexpr int MIR = (2 * R + 3) & ~3;           // mirrored ring head
    static_assert(C + N + GW <= RING, "jump ring too small");
    static_assert(MIR <= RING, "mirror longer than the ring");
    template <typename W>
    __host__ __device__ static constexpr size_t bytes(int nwords) {
        return sizeof(W) * (size_t)(2 * NJ + RING + MIR) +
               sizeof(uint32_t) * (size_t)(nwords + PAD);
    }
};

// Ring slot k (k < RING) written with its mirror copy.
template <class Geo, typename W>
__device__ __forceinline__ void ringPut(W *ring, uint32_t k, W v) {
    ring[k] = v;
    if (k < (uint32_t)Geo::MIR) ring[Geo::RING + k] = v;
}

// The taps of one group, J .. J+3, against the lane's R outputs: bit t of
// D says whether tap J + t is set.  Tap J + t reads seq[base + J + t + r]
// for output r: win[(J + t + r) % R] while t + r < R (the register window,
// rotated), else nx[t + r - R], the words just past the window.  The terms
// are XOR-ed in a chain that the compiler fuses into three-input XORs (two
// terms per instruction).
template <class Tr, int R, int J, int D>
__device__ __forceinline__ void tapGroup(typename Tr::W (&acc)[R], const typename Tr::W (&win)[R],
                                         const typename Tr::W (&nx)[4]) {
    using W = typename Tr::W;
#pragma unroll
    for (int r = 0; r < R; r++) {
        W v = acc[r];
#pragma unroll
        for (int t = 0; t < 4; t++)
            if ((D >> t) & 1) v ^= (t + r < R) ? win[(J + t + r) % R] : nx[t + r - R];
        acc[r] = v;
    }
}

// One uniform branch per group of NT4 <= 4 taps: the group's coefficient
// bits are the same for the whole warp.
template <class Tr, int R, int J, int NT4>
__device__ __forceinline__ void tapSwitch(typename Tr::W (&acc)[R], const typename Tr::W (&win)[R],
                                          const typename Tr::W (&nx)[4], uint32_t d) {
#define MTGP_TAP_CASE(D) \
    case D:              \
        if constexpr ((D >> NT4) == 0) tapGroup<Tr, R, J, D>(acc, win, nx); \
        break;
    switch (d) {
        MTGP_TAP_CASE(1) MTGP_TAP_CASE(2) MTGP_TAP_CASE(3) MTGP_TAP_CASE(4)
        MTGP_TAP_CASE(5) MTGP_TAP_CASE(6) MTGP_TAP_CASE(7) MTGP_TAP_CASE(8)
        MTGP_TAP_CASE(9) MTGP_TAP_CASE(10) MTGP_TAP_CASE(11) MTGP_TAP_CASE(12)
        MTGP_TAP_CASE(13) MTGP_TAP_CASE(14) MTGP_TAP_CASE(15)
    default: break;
    }
#undef MTGP_TAP_CASE
}

// Groups J, J + 4, ... of the R taps of one tapsR call; each group's words
// replace the window words its taps no longer need.
template <class Tr, int R, int J>
__device__ __forceinline__ void tapGroups(typename Tr::W (&acc)[R], typename Tr::W (&win)[R],
                                          const typename Tr::W *rp, uint32_t bits_lo,
                                          uint32_t bits_hi) {
    if constexpr (J < R) {
        using W = typename Tr::W;
        constexpr int NT4 = R - J < 4 ? R - J : 4;
        const uint32_t bj = J < 32 ? bits_lo : bits_hi;  // J % 4 == 0: never straddles bit 31
        const uint32_t d = (bj >> (J & 31)) & ((1u << NT4) - 1u);
        W nx[4];
#pragma unroll
        for (int u = 0; u < 4; u++) nx[u] = u < NT4 ? rp[R + J + u] : W(0);
        tapSwitch<Tr, R, J, NT4>(acc, win, nx, d);
#pragma unroll
        for (int u = 0; u < NT4; u++) win[J + u] = nx[u];
        tapGroups<Tr, R, J + 4>(acc, win, rp, bits_lo, bits_hi);
    }
}

// Largest R for which taps go in groups of four (a 16-way branch per group,
// whose code grows with R); larger R take them in pairs.  Groups of four
// hold a few more registers live, so the jumps inside the batched kernels
// (whose generation core caps the registers) keep pairs.
constexpr int kQuadTapsMaxR = 13;

// R taps p .. p+R-1 against the lane's R outputs: win holds seq[p + l0 ..
// + R) on entry (l0 folded into base = p + l0) and the next R words on exit.
// rp = ring + (base & (RING - 1)): the next R words are rp[R .. 2R), which
// the mirror keeps contiguous, so every load is one base plus a constant.
// The coefficients of a group of taps are the same for the whole warp, so
// each group takes one uniform branch.  In groups of four, a set of m taps
// costs ceil(m / 2) three-input XORs per output (1.25 per group on random
// polynomials, 0.31 per tap); in pairs (larger R) 0.375 per tap.
template <class Tr, class Geo, bool GROUPS4>
__device__ __forceinline__ void tapsR(typename Tr::W (&acc)[Geo::R], typename Tr::W (&win)[Geo::R],
                                      const typename Tr::W *rp, uint32_t bits_lo,
                                      uint32_t bits_hi) {
    constexpr int R = Geo::R;
    if constexpr (GROUPS4 && R <= kQuadTapsMaxR) {
        tapGroups<Tr, R, 0>(acc, win, rp, bits_lo, bits_hi);
    } else {
#pragma unroll
    for (int j = 0; j < R; j += 2) {  // j even: a pair never straddles bit 31
        const uint32_t bj = j < 32 ? bits_lo : bits_hi;
        if (j + 1 < R) {
            // tap j reads seq[base + j .. + R) = win[(j + r) % R]; tap j + 1
            // reads seq[base + j + 1 .. + R), whose last word is the one that
            // replaces win[j]
            const typename Tr::W next = rp[R + j];
            auto w1 = [&](int r) { return r < R - 1 ? win[(j + 1 + r) % R] : next; };
            const uint32_t b2 = (bj >> (j & 31)) & 3u;
            if (b2 == 3u) {
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] ^= win[(j + r) % R] ^ w1(r);
            } else if (b2 == 1u) {
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] ^= win[(j + r) % R];
            } else if (b2 == 2u) {
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] ^= w1(r);
            }
            win[j] = next;
            win[j + 1] = rp[R + j + 1];
        } else {  // the last tap of an odd R, on its own
            if ((bj >> (j & 31)) & 1u) {
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] ^= win[(j + r) % R];
            }
            win[j] = rp[R + j];
        }
    }
    }
}

// Jump the window jin[0..N) in place by chain[0], chain[1], ... (uint32-array
// polynomials of nwords words).  smem must hold Geo::bytes<W>(nwords) bytes
// laid out as described above (jin first).  All NT threads must call it; it
// begins and ends with a barrier.  GROUPS4: taps in groups of four (tapsR).
template <class Tr, class Geo, bool GROUPS4, class ChainAt>
__device__ __forceinline__ void jump_chain_impl(typename Tr::W *smem, const typename Tr::Lane &L,
                                                ChainAt chain, int nchain, int nwords) {
    using W = typename Tr::W;
    constexpr int N = Geo::N, R = Geo::R, NT = Geo::NT;
    constexpr uint32_t M = Geo::RING - 1;
    W *jin = smem;
    W *jout = jin + Geo::NJ;
    W *ring = jout + Geo::NJ;
    uint32_t *poly = reinterpret_cast<uint32_t *>(ring + Geo::RING + Geo::MIR);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int taps = nwords * 32;
    const int pwords = nwords + Geo::PAD;
    __syncthreads();

    for (int c = 0; c < nchain; c++) {
        const uint32_t *pg = chain(c);
        for (int k = tid; k < pwords; k += NT) poly[k] = k < nwords ? pg[k] : 0u;
        for (int k = tid; k < N; k += NT) jout[k] = 0;
        for (int g = 0; g < Geo::G; g++) {
            for (int k = tid; k < N; k += NT) ringPut<Geo>(ring, (uint32_t)k, jin[k]);
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
                        ringPut<Geo>(ring, w & M, Tr::rec(x1, x2, y, L));
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
                    tapsR<Tr, Geo, GROUPS4>(acc, win, ring + ((uint32_t)(p + l0) & M), bits_lo, bits_hi);
                }
                __syncthreads();
            }
#pragma unroll
            for (int r = 0; r < R; r++)
                if (l0 + r < N) Tr::axor(&jout[l0 + r], acc[r]);
            __syncthreads();
        }
        for (int k = tid; k < N; k += NT) jin[k] = jout[k];
        __syncthreads();
    }
}

template <class Tr, class Geo>
__device__ void jump_chain(typename Tr::W *smem, const typename Tr::Lane &L,
                           const uint32_t *const *chain, int nchain, int nwords) {
    jump_chain_impl<Tr, Geo, true>(smem, L, [chain](int c) { return chain[c]; }, nchain, nwords);
}

// One polynomial.
template <class Tr, class Geo>
__device__ void jump_one(typename Tr::W *smem, const typename Tr::Lane &L, const uint32_t *poly,
                         int nwords) {
    jump_chain_impl<Tr, Geo, true>(smem, L, [poly](int) { return poly; }, 1, nwords);
}

// Part of one jump: the correlation over the tap chunks [ch0, ch1) only
// (chunks of Geo::C taps), XOR-ed into gdst[0..N) in global memory with
// atomicXor (gdst must start at zero; the parts of one jump may run in any
// order on any CTAs).  smem holds the window in jin on entry.  The recursion
// is still generated from the window up to the last tap of the range.
template <class Tr, class Geo>
__device__ void jump_part(typename Tr::W *smem, const typename Tr::Lane &L, const uint32_t *pg,
                          int nwords, int ch0, int ch1, typename Tr::W *gdst) {
    using W = typename Tr::W;
    constexpr int N = Geo::N, R = Geo::R, NT = Geo::NT;
    constexpr uint32_t M = Geo::RING - 1;
    W *jin = smem;
    W *ring = jin + 2 * Geo::NJ;
    uint32_t *poly = reinterpret_cast<uint32_t *>(ring + Geo::RING + Geo::MIR);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int pwords = nwords + Geo::PAD;
    for (int k = tid; k < pwords; k += NT) poly[k] = k < nwords ? pg[k] : 0u;
    for (int g = 0; g < Geo::G; g++) {
        for (int k = tid; k < N; k += NT) ringPut<Geo>(ring, (uint32_t)k, jin[k]);
        __syncthreads();
        int generated = N;
        const int l0 = g * 32 * R + lane * R;
        W acc[R];
#pragma unroll
        for (int r = 0; r < R; r++) acc[r] = 0;
        for (int ch = 0; ch < ch1; ch++) {
            const int cs = ch * Geo::C;
            while (generated < cs + Geo::C + N) {
                if (tid < Geo::GW) {
                    uint32_t w = (uint32_t)(generated + tid);
                    W x1 = ring[(w - N) & M];
                    W x2 = ring[(w - N + 1) & M];
                    W y = ring[(w - N + L.pos) & M];
                    ringPut<Geo>(ring, w & M, Tr::rec(x1, x2, y, L));
                }
                __syncthreads();
                generated += Geo::GW;
            }
            if (ch >= ch0) {
                const int i0 = cs + warp * Geo::TPW;
                W win[R];
#pragma unroll
                for (int r = 0; r < R; r++) win[r] = ring[(uint32_t)(i0 + l0 + r) & M];
                for (int jb = 0; jb < Geo::TPW; jb += R) {
                    const int p = i0 + jb;
                    const uint32_t bits_lo =
                        __funnelshift_r(poly[p >> 5], poly[(p >> 5) + 1], p & 31);
                    const uint32_t bits_hi =
                        R > 32 ? __funnelshift_r(poly[(p >> 5) + 1], poly[(p >> 5) + 2], p & 31)
                               : 0u;
                    tapsR<Tr, Geo, true>(acc, win, ring + ((uint32_t)(p + l0) & M), bits_lo, bits_hi);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int r = 0; r < R; r++)
            if (l0 + r < N) Tr::axor(&gdst[l0 + r], acc[r]);
        __syncthreads();
    }
}

}  // namespace mtgp
