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

// Squaring in GF(2)[x] spreads the bits: coefficient i moves to 2i.
Poly sqrmod(const Poly &a, const Poly &m, int dm) {
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
    reduce(r, m, dm);
    return r;
}

Poly powxmod(const std::vector<uint32_t> &e, const Poly &m, int dm) {
    const int W = (dm + 63) / 64;
    Poly r(W, 0);
    r[0] = 1;
    int top = (int)e.size() * 32 - 1;
    while (top >= 0 && !((e[top / 32] >> (top % 32)) & 1u)) top--;
    for (int i = top; i >= 0; i--) {
        r = sqrmod(r, m, dm);
        if ((e[i / 32] >> (i % 32)) & 1u) {
            // r *= X
            Poly t(W + 1, 0);
            for (int k = 0; k < W; k++) {
                t[k] ^= r[k] << 1;
                t[k + 1] ^= r[k] >> 63;
            }
            reduce(t, m, dm);
            r = t;
        }
    }
    r.resize(W);
    return r;
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
