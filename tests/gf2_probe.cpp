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
