// gf2_probe.cpp -- C entry points over the library's host GF(2)[x] code
// (mtgp_gb300/csrc/gf2.cpp), compiled by tests/test_gf2_host.py so that the
// jump-polynomial arithmetic can be checked against the oracle on the CPU.
#include <cstring>

#include "../mtgp_gb300/csrc/gf2.h"

using mtgp::gf2::Modulus;
using mtgp::gf2::Poly;

static Poly take(const uint64_t *w, int n) { return Poly(w, w + n); }

extern "C" {

// X^e mod m (m: dm/64+1 words); out: (dm+63)/64 words.
int probe_powx(const uint64_t *m, int dm, const uint32_t *e, int ew, uint64_t *out) {
    Modulus M(take(m, dm / 64 + 1), dm);
    Poly r = M.powx(std::vector<uint32_t>(e, e + ew));
    std::memcpy(out, r.data(), sizeof(uint64_t) * M.words());
    return 0;
}

// a * b mod m (a, b: (dm+63)/64 words).
int probe_mulmod(const uint64_t *a, const uint64_t *b, const uint64_t *m, int dm, uint64_t *out) {
    Modulus M(take(m, dm / 64 + 1), dm);
    Poly r = M.mulmod(take(a, M.words()), take(b, M.words()));
    std::memcpy(out, r.data(), sizeof(uint64_t) * M.words());
    return 0;
}

// X^e mod m as the product of X^(2^i) over the set bits of a 64-bit e
// (the way batched plans build their jump polynomials).
int probe_pow2_product(const uint64_t *m, int dm, uint64_t e, uint64_t *out) {
    Modulus M(take(m, dm / 64 + 1), dm);
    Poly x((size_t)M.words(), 0), r;
    x[0] = 2;
    for (int i = 0; i < 64; i++) {
        if ((e >> i) & 1u) r = r.empty() ? x : M.mulmod(r, x);
        x = M.sqrmod(x);
    }
    if (r.empty()) {
        r.assign((size_t)M.words(), 0);
        r[0] = 1;
    }
    std::memcpy(out, r.data(), sizeof(uint64_t) * M.words());
    return 0;
}
}

// floor(X^e / m): quotient words into out ((e - dm) / 64 + 1 words).
extern "C" int probe_divxpow(const uint64_t *m, int dm, int e, uint64_t *out) {
    Poly q = mtgp::gf2::divXpow(e, take(m, dm / 64 + 1), dm);
    std::memcpy(out, q.data(), sizeof(uint64_t) * q.size());
    return (int)q.size();
}

#include "../mtgp_gb300/csrc/pow_sched.h"

// X^e[j] mod m for j < n by the GPU's schedules (pow_sched.h), run here with
// the host's products: byte-window table by tableSchedule, then powSchedule
// with `width` concurrent CTAs.  out: n x (dm+63)/64 words; shape: levels,
// steps, scratch slots of the exponent schedule.
extern "C" int probe_pow_schedule(const uint64_t *m, int dm, const uint64_t *e, int n, int width,
                                  uint64_t *out, int *shape) {
    Modulus M(take(m, dm / 64 + 1), dm);
    const size_t w = (size_t)M.words();
    std::vector<Poly> tab(mtgp::kPowSlots);
    Poly x(w, 0);
    x[0] = 2;
    for (int i = 0; i < 64; i++) {
        tab[(size_t)mtgp::powSlot(i / 8, 1 << (i % 8))] = x;
        x = M.sqrmod(x);
    }
    Poly one(w, 0);
    one[0] = 1;
    std::vector<Poly> scratch, res((size_t)n);
    auto run = [&](const mtgp::PowSchedule &s, std::vector<Poly> &dst) {
        for (const auto &lev : s.levels) {
            std::vector<std::pair<const mtgp::PowStep *, Poly>> done;
            for (const mtgp::PowStep &st : lev) {  // all reads before any write
                Poly r = one;
                for (int k = 0; k < st.nsrc; k++) {
                    const int c = st.src[k];
                    const Poly &f = c >= 0 ? tab[(size_t)c] : scratch.at((size_t)(-1 - c));
                    if (f.empty()) return -1;  // a slot read before it was made
                    r = k == 0 ? f : M.mulmod(r, f);
                }
                done.emplace_back(&st, r);
            }
            for (auto &d : done) {
                if (d.first->dst >= 0)
                    dst.at((size_t)d.first->dst) = d.second;
                else
                    scratch.at((size_t)(-1 - d.first->dst)) = d.second;
            }
        }
        return 0;
    };
    mtgp::PowSchedule ts;
    mtgp::tableSchedule(ts);
    if (run(ts, tab)) return -1;
    mtgp::PowSchedule s;
    mtgp::powSchedule(e, n, width, s);
    scratch.assign((size_t)s.nscratch, Poly());
    if (run(s, res)) return -2;
    for (int j = 0; j < n; j++) {
        if (res[(size_t)j].size() != w) return -3;
        std::memcpy(out + (size_t)j * w, res[(size_t)j].data(), sizeof(uint64_t) * w);
    }
    shape[0] = (int)s.levels.size();
    shape[1] = s.steps();
    shape[2] = s.nscratch;
    return 0;
}

// The GPU kernels' formulations (bm_kernels.cu), restated serially with the
// same 32-bit word layout:
//   probe_bm_reversed: Berlekamp-Massey where the discrepancy at step N is
//     the parity of C AND (R >> (n2 - 1 - N)), R the bit-reversed sequence;
//     out = chi (the reciprocal of C) in 64-bit words, returns L;
//   probe_barrett_series: mu = floor(X^(2D) / chi) as the power series
//     1 / C(x) to D + 1 terms stored reversed.
namespace {
uint32_t wordAt(const std::vector<uint32_t> &v, long w) {
    return (w >= 0 && w < (long)v.size()) ? v[(size_t)w] : 0u;
}
uint32_t shr32(const std::vector<uint32_t> &v, long w, long sh) {
    const long q = w + (sh >> 5);
    const int b = (int)(sh & 31);
    const uint64_t lo = wordAt(v, q), hi = wordAt(v, q + 1);
    return (uint32_t)(((hi << 32) | lo) >> b);
}
uint32_t shl32(const std::vector<uint32_t> &v, long w, long sh) {
    const long q = w - (sh >> 5);
    const int b = (int)(sh & 31);
    const uint64_t lo = wordAt(v, q - 1), hi = wordAt(v, q);
    return (uint32_t)((((hi << 32) | lo) << b) >> 32);
}
}  // namespace

extern "C" int probe_bm_reversed(const uint8_t *s, int n2, uint64_t *chi_out) {
    const int nr = (n2 + 31) / 32 + 2, nw = n2 / 64 + 2;
    std::vector<uint32_t> R((size_t)nr, 0), C((size_t)nw, 0), B((size_t)nw, 0), T((size_t)nw, 0);
    for (int k = 0; k < n2; k++)
        if (s[n2 - 1 - k] & 1) R[(size_t)k >> 5] |= 1u << (k & 31);
    C[0] = B[0] = 1;
    int L = 0, m = -1;
    for (int N = 0; N < n2; N++) {
        const int base = n2 - 1 - N, lw = L / 32 + 1;
        uint32_t acc = 0;
        for (int w = 0; w < lw; w++) acc ^= C[(size_t)w] & shr32(R, w, base);
        if (!(__builtin_popcount(acc) & 1)) continue;
        const int sh = N - m;
        const bool grow = 2 * L <= N;
        const int nl = grow ? N + 1 - L : L, top = (nl > L ? nl : L) / 32 + 1;
        if (grow) {
            for (int w = 0; w < nw; w++)
                T[(size_t)w] = w < top ? C[(size_t)w] ^ shl32(B, w, sh) : 0u;
            std::swap(B, C);   // B = old C
            std::swap(C, T);   // C = new
            L = nl;
            m = N;
        } else {
            std::vector<uint32_t> add((size_t)top);
            for (int w = 0; w < top && w < nw; w++) add[(size_t)w] = shl32(B, w, sh);
            for (int w = 0; w < top && w < nw; w++) C[(size_t)w] ^= add[(size_t)w];
        }
    }
    for (int i = 0; i <= L; i++) {
        const int q = L - i;
        if ((C[(size_t)q >> 5] >> (q & 31)) & 1u) chi_out[i >> 6] |= 1ULL << (i & 63);
    }
    return L;
}

extern "C" int probe_barrett_series(const uint64_t *m, int D, uint64_t *mu_out) {
    const int nw = D / 32 + 1;
    std::vector<uint32_t> chi((size_t)nw, 0), Cp((size_t)nw, 0), Z((size_t)nw + 2, 0);
    for (int i = 0; i <= D; i++)
        if ((m[i >> 6] >> (i & 63)) & 1u) chi[(size_t)i >> 5] |= 1u << (i & 31);
    for (int i = 0; i < D; i++)  // C' bit i = C_{i+1} = chi_{D-1-i}
        if ((chi[(size_t)(D - 1 - i) >> 5] >> ((D - 1 - i) & 31)) & 1u)
            Cp[(size_t)i >> 5] |= 1u << (i & 31);
    Z[(size_t)D >> 5] |= 1u << (D & 31);
    for (int k = 1; k <= D; k++) {
        const int base = D - k + 1, lw = (k - 1) / 32 + 1;
        uint32_t acc = 0;
        for (int w = 0; w < lw; w++) acc ^= Cp[(size_t)w] & shr32(Z, w, base);
        if (__builtin_popcount(acc) & 1) Z[(size_t)(D - k) >> 5] |= 1u << ((D - k) & 31);
    }
    for (int i = 0; i <= D; i++)
        if ((Z[(size_t)i >> 5] >> (i & 31)) & 1u) mu_out[i >> 6] |= 1ULL << (i & 63);
    return 0;
}
