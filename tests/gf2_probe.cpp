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
