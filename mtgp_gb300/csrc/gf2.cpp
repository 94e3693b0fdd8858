// gf2.cpp -- word-level GF(2)[x] arithmetic (see gf2.h).
#include "gf2.h"

#include <algorithm>
#include <cctype>

namespace mtgp {
namespace gf2 {

int degree(const Poly &p) {
    for (int k = (int)p.size() - 1; k >= 0; k--)
        if (p[k]) return 64 * k + 63 - __builtin_clzll(p[k]);
    return -1;
}

// 64x64 -> 128-bit carry-less product, 4-bit windows (portable).
static inline void clmul64(uint64_t a, uint64_t b, uint64_t *lo, uint64_t *hi) {
    uint64_t tl[16], th[16];
    tl[0] = th[0] = 0;
    tl[1] = a;
    th[1] = 0;
    for (int i = 2; i < 16; i += 2) {
        tl[i] = tl[i / 2] << 1;
        th[i] = (th[i / 2] << 1) | (tl[i / 2] >> 63);
        tl[i + 1] = tl[i] ^ a;
        th[i + 1] = th[i];
    }
    uint64_t l = 0, h = 0;
    for (int s = 60; s >= 0; s -= 4) {
        // (h:l) <<= 4, then xor the window product
        h = (h << 4) | (l >> 60);
        l <<= 4;
        unsigned v = (unsigned)(b >> s) & 15u;
        l ^= tl[v];
        h ^= th[v];
    }
    *lo = l;
    *hi = h;
}

Poly mul(const Poly &a, const Poly &b) {
    Poly r(a.size() + b.size() + 1, 0);
    for (size_t i = 0; i < a.size(); i++) {
        if (!a[i]) continue;
        for (size_t j = 0; j < b.size(); j++) {
            if (!b[j]) continue;
            uint64_t lo, hi;
            clmul64(a[i], b[j], &lo, &hi);
            r[i + j] ^= lo;
            r[i + j + 1] ^= hi;
        }
    }
    return r;
}

// p ^= m << shift over the words of p.
static inline void xorShifted(Poly &p, const Poly &m, int mwords, int shift) {
    int ws = shift >> 6, bs = shift & 63;
    for (int k = 0; k < mwords; k++) {
        size_t d = (size_t)(k + ws);
        if (d >= p.size()) break;
        p[d] ^= m[k] << bs;
        if (bs && d + 1 < p.size()) p[d + 1] ^= m[k] >> (64 - bs);
    }
}

void reduce(Poly &p, const Poly &m, int dm) {
    const int mwords = dm / 64 + 1;
    for (int i = degree(p); i >= dm; i--) {
        if ((p[i >> 6] >> (i & 63)) & 1u) xorShifted(p, m, mwords, i - dm);
    }
    p.resize((size_t)(dm + 63) / 64);
}

Poly mulmod(const Poly &a, const Poly &b, const Poly &m, int dm) {
    Poly r = mul(a, b);
    reduce(r, m, dm);
    return r;
}

static Poly spread(const Poly &a);

Poly sqrmod(const Poly &a, const Poly &m, int dm) {
    Poly r = spread(a);
    reduce(r, m, dm);
    return r;
}

// Spread the bits of a: coefficient i moves to 2i (squaring in GF(2)[x]).
static Poly spread(const Poly &a) {
    Poly r(2 * a.size() + 1, 0);
    for (size_t k = 0; k < a.size(); k++) {
        uint64_t x = a[k];
        for (int h = 0; h < 2; h++) {
            uint64_t v = (x >> (32 * h)) & 0xffffffffu;
            v = (v | (v << 16)) & 0x0000ffff0000ffffULL;
            v = (v | (v << 8)) & 0x00ff00ff00ff00ffULL;
            v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0fULL;
            v = (v | (v << 2)) & 0x3333333333333333ULL;
            v = (v | (v << 1)) & 0x5555555555555555ULL;
            r[2 * k + h] = v;
        }
    }
    return r;
}

Poly mulComb(const Poly &a, const Poly &b) {
    const size_t tw = b.size() + 1;
    // t[v] = v(X) * b(X) for every byte v
    std::vector<uint64_t> t(256 * tw, 0);
    for (int i = 0; i < 8; i++) {
        uint64_t *d = &t[(size_t)(1u << i) * tw];
        for (size_t k = 0; k < b.size(); k++) {
            d[k] ^= b[k] << i;
            if (i) d[k + 1] ^= b[k] >> (64 - i);
        }
    }
    for (unsigned v = 3; v < 256; v++) {
        const unsigned lo = v & (0u - v);
        if (lo == v) continue;
        const uint64_t *x = &t[(size_t)lo * tw], *y = &t[(size_t)(v ^ lo) * tw];
        uint64_t *d = &t[(size_t)v * tw];
        for (size_t k = 0; k < tw; k++) d[k] = x[k] ^ y[k];
    }
    // comb: byte k of every word of a, from the top byte down, shifting the
    // partial product by 8 between bytes
    Poly r(a.size() + tw, 0);
    for (int k = 7; k >= 0; k--) {
        for (size_t i = 0; i < a.size(); i++) {
            const unsigned v = (unsigned)(a[i] >> (8 * k)) & 255u;
            if (!v) continue;
            const uint64_t *x = &t[(size_t)v * tw];
            uint64_t *d = &r[i];
            for (size_t q = 0; q < tw; q++) d[q] ^= x[q];
        }
        if (k)
            for (size_t q = r.size() - 1; q > 0; q--) r[q] = (r[q] << 8) | (r[q - 1] >> 56);
        if (k) r[0] <<= 8;
    }
    return r;
}

Modulus::Modulus(const Poly &m, int dm) : m_(m), dm_(dm) {
    m_.resize((size_t)dm / 64 + 1, 0);
    tw_ = dm / 64 + 2;
    // coefficients dm-1 .. dm-7 of m: mrev bit 7-i = coefficient dm-i
    unsigned mrev = 0;
    for (int i = 0; i <= 7; i++) {
        const int c = dm - i;
        if (c >= 0 && ((m_[(size_t)c >> 6] >> (c & 63)) & 1u)) mrev |= 1u << (7 - i);
    }
    tab_.assign((size_t)8 * 256 * tw_, 0);
    for (unsigned b = 1; b < 256; b++) {
        // quotient q clearing coefficients dm..dm+7 (= b) from the top
        unsigned res = b, q = 0;
        for (int k = 7; k >= 0; k--) {
            if (!((res >> k) & 1u)) continue;
            q |= 1u << k;
            res ^= mrev >> (7 - k);  // m * X^k touches window bits k, k-1, ..., 0
        }
        uint64_t *d = &tab_[(size_t)b * tw_];  // alignment 0
        for (int i = 0; i < 8; i++) {
            if (!((q >> i) & 1u)) continue;
            for (size_t k = 0; k < m_.size(); k++) {
                d[k] ^= m_[k] << i;
                if (i) d[k + 1] ^= m_[k] >> (64 - i);
            }
        }
        for (int a = 1; a < 8; a++) {  // the same entry shifted by 8a bits
            uint64_t *e = &tab_[((size_t)a * 256 + b) * tw_];
            const int sh = 8 * a;
            for (int k = 0; k < tw_; k++) {
                e[k] = d[k] << sh;
                if (k) e[k] |= d[k - 1] >> (64 - sh);
            }
        }
    }
}

void Modulus::reduce(Poly &p) const {
    const int D = gf2::degree(p);
    if (D >= dm_) {
        for (int t = (D - dm_) / 8; t >= 0; t--) {
            const int j = dm_ + 8 * t;  // window of coefficients j .. j+7
            const size_t w = (size_t)j >> 6;
            const int o = j & 63;
            uint64_t v = p[w] >> o;
            if (o > 56 && w + 1 < p.size()) v |= p[w + 1] << (64 - o);
            const unsigned b = (unsigned)v & 255u;
            if (!b) continue;
            const int s = 8 * t;  // the entry lands at coefficient s
            const uint64_t *x = &tab_[((size_t)((s & 63) >> 3) * 256 + b) * tw_];
            const size_t ws = (size_t)s >> 6;
            const size_t n = std::min(p.size() - ws, (size_t)tw_);
            uint64_t *d = &p[ws];
            for (size_t k = 0; k < n; k++) d[k] ^= x[k];
        }
    }
    p.resize((size_t)words(), 0);
}

Poly Modulus::mulmod(const Poly &a, const Poly &b) const {
    Poly r = mulComb(a, b);
    reduce(r);
    return r;
}

Poly Modulus::sqrmod(const Poly &a) const {
    Poly r = spread(a);
    reduce(r);
    return r;
}

Poly Modulus::powx(const std::vector<uint32_t> &e) const {
    const int W = words();
    Poly r(W, 0);
    r[0] = 1;
    int top = (int)e.size() * 32 - 1;
    while (top >= 0 && !((e[top / 32] >> (top % 32)) & 1u)) top--;
    for (int i = top; i >= 0; i--) {
        r = sqrmod(r);
        if ((e[i / 32] >> (i % 32)) & 1u) {  // r *= X
            Poly t(W + 1, 0);
            for (int k = 0; k < W; k++) {
                t[k] ^= r[k] << 1;
                t[k + 1] ^= r[k] >> 63;
            }
            reduce(t);
            r.swap(t);
        }
    }
    return r;
}

Poly divXpow(int e, const Poly &m, int dm) {
    // remainder r starts as X^e; clear its bits from the top with shifted m
    Poly r((size_t)e / 64 + 1, 0), q((size_t)(e - dm) / 64 + 1, 0);
    r[(size_t)e >> 6] = uint64_t(1) << (e & 63);
    const int mw = dm / 64 + 1;
    for (int b = e; b >= dm; b--) {
        if (!((r[(size_t)b >> 6] >> (b & 63)) & 1u)) continue;
        const int sh = b - dm;
        q[(size_t)sh >> 6] |= uint64_t(1) << (sh & 63);
        const int ws = sh >> 6, bs = sh & 63;
        for (int k = 0; k < mw; k++) {
            const size_t d = (size_t)(k + ws);
            if (d >= r.size()) break;
            r[d] ^= m[(size_t)k] << bs;
            if (bs && d + 1 < r.size()) r[d + 1] ^= m[(size_t)k] >> (64 - bs);
        }
    }
    return q;
}

Poly powxmod(const std::vector<uint32_t> &e, const Poly &m, int dm) {
    return Modulus(m, dm).powx(e);
}

// Berlekamp-Massey over GF(2) with word-parallel discrepancy: the last L bits
// of s are kept reversed in a register file so that d = parity(C & S).
int minpoly(const std::vector<uint8_t> &s, Poly *chi) {
    const int n = (int)s.size();
    const int W = n / 64 + 2;
    Poly C(W, 0), B(W, 0), T(W, 0), S(W, 0);
    C[0] = B[0] = 1;
    int L = 0, m = -1;
    for (int N = 0; N < n; N++) {
        // S bit i = s[N - i] for i >= 0 (bit 0 = current sample)
        for (int k = W - 1; k > 0; k--) S[k] = (S[k] << 1) | (S[k - 1] >> 63);
        S[0] = (S[0] << 1) | (uint64_t)(s[N] & 1);
        uint64_t acc = 0;
        const int lw = L / 64 + 1;
        for (int k = 0; k < lw && k < W; k++) acc ^= C[k] & S[k];
        int d = __builtin_parityll(acc);
        if (!d) continue;
        T = C;
        int shift = N - m;
        int ws = shift >> 6, bs = shift & 63;
        for (int k = W - 1; k >= 0; k--) {
            uint64_t v = 0;
            int src = k - ws;
            if (src >= 0) {
                v = B[src] << bs;
                if (bs && src - 1 >= 0) v |= B[src - 1] >> (64 - bs);
            }
            C[k] ^= v;
        }
        if (2 * L <= N) {
            L = N + 1 - L;
            m = N;
            B = T;
        }
    }
    Poly out((size_t)L / 64 + 1, 0);
    for (int i = 0; i <= L; i++) {
        int j = L - i;
        if ((C[j >> 6] >> (j & 63)) & 1u) out[i >> 6] |= 1ULL << (i & 63);
    }
    *chi = out;
    return L;
}

std::vector<uint32_t> toWords32(const Poly &p, int nwords) {
    std::vector<uint32_t> w((size_t)nwords, 0);
    for (int k = 0; k < nwords; k++) {
        size_t q = (size_t)k / 2;
        if (q < p.size()) w[k] = (uint32_t)(p[q] >> (32 * (k & 1)));
    }
    return w;
}

Poly fromWords32(const uint32_t *w, int nwords) {
    Poly p((size_t)(nwords + 1) / 2, 0);
    for (int k = 0; k < nwords; k++) p[k / 2] |= (uint64_t)w[k] << (32 * (k & 1));
    return p;
}

bool fromHex(const char *s, Poly *p, int *ncoef) {
    size_t len = 0;
    while (s[len]) len++;
    Poly r(len * 4 / 64 + 1, 0);
    for (size_t k = 0; k < len; k++) {
        int ch = (unsigned char)s[k];
        if (!std::isxdigit(ch)) return false;
        ch = std::tolower(ch);
        uint64_t v = (uint64_t)(ch >= 'a' ? ch - 'a' + 10 : ch - '0');
        size_t bit = 4 * k;
        r[bit >> 6] |= v << (bit & 63);  // 4-bit groups never straddle words
    }
    *p = r;
    if (ncoef) *ncoef = (int)(len * 4);
    return true;
}

std::string toHex(const Poly &p) {
    static const char dig[] = "0123456789abcdef";
    int d = degree(p);
    std::string s;
    for (int k = 0; k <= d / 4; k++) s.push_back(dig[(p[(4 * k) >> 6] >> ((4 * k) & 63)) & 15]);
    return s;
}

}  // namespace gf2
}  // namespace mtgp
