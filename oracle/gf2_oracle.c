/*
 * gf2_oracle.c -- bit-serial GF(2)[x] arithmetic for the test oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see mtgp_oracle.h).  The reference computes its
 * characteristic polynomials with NTL's MinPolySeq over 2*mexp output LSBs
 * (mtgp32-calc-poly.cpp:36-45) and its jump polynomials with NTL's PowerXMod
 * (mtgp-calc-jump.hpp:135-162); NTL is not part of the reference tree.  This
 * file restates the published algorithms: Berlekamp-Massey over GF(2), and
 * left-to-right square-and-multiply for X^e mod m.  It is written for
 * obviousness, not speed.
 */
#include "mtgp_oracle.h"

#include <ctype.h>
#include <stdlib.h>
#include <string.h>

static inline int getb(const uint64_t *p, int i) {
    return (int)((p[i >> 6] >> (i & 63)) & 1u);
}
static inline void flipb(uint64_t *p, int i) { p[i >> 6] ^= UINT64_C(1) << (i & 63); }

/* dst ^= src << shift, dst has dwords words (bits beyond are dropped). */
static void xor_shl(uint64_t *dst, int dwords, const uint64_t *src, int swords,
                    int shift) {
    int ws = shift >> 6, bs = shift & 63;
    for (int k = 0; k < swords; k++) {
        int d = k + ws;
        if (d >= dwords) break;
        dst[d] ^= src[k] << bs;
        if (bs && d + 1 < dwords) dst[d + 1] ^= src[k] >> (64 - bs);
    }
}

/* Berlekamp-Massey over GF(2) (Massey 1969).  Returns L and writes the
 * minimal polynomial chi (degree L, monic), the reciprocal of the connection
 * polynomial, which is NTL MinPolySeq's convention. */
int orc_gf2_minpoly(const uint8_t *bits, int n, uint64_t *out, int nwords) {
    int W = n / 64 + 2;
    uint64_t *C = (uint64_t *)calloc((size_t)W, 8);
    uint64_t *B = (uint64_t *)calloc((size_t)W, 8);
    uint64_t *T = (uint64_t *)calloc((size_t)W, 8);
    C[0] = 1;
    B[0] = 1;
    int L = 0, m = -1;
    for (int N = 0; N < n; N++) {
        int d = bits[N] & 1;
        for (int i = 1; i <= L; i++)
            if (getb(C, i)) d ^= bits[N - i] & 1;
        if (!d) continue;
        memcpy(T, C, (size_t)W * 8);
        xor_shl(C, W, B, W, N - m);
        if (2 * L <= N) {
            L = N + 1 - L;
            m = N;
            memcpy(B, T, (size_t)W * 8);
        }
    }
    memset(out, 0, (size_t)nwords * 8);
    for (int i = 0; i <= L; i++)
        if (getb(C, L - i) && (i >> 6) < nwords) flipb(out, i);
    free(C);
    free(B);
    free(T);
    return L;
}

/* r = r * X mod m (r has degree < dm). */
static void mulx_mod(uint64_t *r, const uint64_t *m, int dm, int W) {
    int carry = 0;
    for (int k = 0; k < W; k++) {
        int c2 = (int)(r[k] >> 63);
        r[k] = (r[k] << 1) | (uint64_t)carry;
        carry = c2;
    }
    if (getb(r, dm)) {
        for (int k = 0; k < W; k++) r[k] ^= m[k];
    }
}

void orc_gf2_mulmod(const uint64_t *a, const uint64_t *b, const uint64_t *m,
                    int dm, uint64_t *out) {
    int W = dm / 64 + 1;             /* room for bit dm during reduction */
    int Wo = (dm + 63) / 64;
    uint64_t *r = (uint64_t *)calloc((size_t)W, 8);
    for (int i = dm - 1; i >= 0; i--) {
        mulx_mod(r, m, dm, W);
        if (getb(b, i))
            for (int k = 0; k < Wo; k++) r[k] ^= a[k];
    }
    memcpy(out, r, (size_t)Wo * 8);
    free(r);
}

void orc_gf2_powxmod(const uint32_t *e, int ewords, const uint64_t *m, int dm,
                     uint64_t *out) {
    int W = dm / 64 + 1;
    int Wo = (dm + 63) / 64;
    uint64_t *r = (uint64_t *)calloc((size_t)W, 8);
    uint64_t *t = (uint64_t *)calloc((size_t)W, 8);
    r[0] = 1;                        /* deg m > 0, so 1 is reduced */
    int top = ewords * 32 - 1;
    while (top >= 0 && !((e[top / 32] >> (top % 32)) & 1u)) top--;
    for (int i = top; i >= 0; i--) {
        orc_gf2_mulmod(r, r, m, dm, t);
        memset(r, 0, (size_t)W * 8);
        memcpy(r, t, (size_t)Wo * 8);
        if ((e[i / 32] >> (i % 32)) & 1u) mulx_mod(r, m, dm, W);
    }
    memcpy(out, r, (size_t)Wo * 8);
    free(r);
    free(t);
}

/* mtgp-calc-jump.hpp:98-126 (stringtopoly): digit k = coefficients 4k..4k+3,
 * least significant bit first. */
int orc_gf2_from_hex(const char *hex, uint64_t *out, int nwords) {
    memset(out, 0, (size_t)nwords * 8);
    int n = 0;
    for (const char *c = hex; *c; c++, n += 4) {
        int ch = (unsigned char)*c;
        if (!isxdigit(ch)) return -1;
        ch = tolower(ch);
        int v = ch >= 'a' ? ch - 'a' + 10 : ch - '0';
        for (int b = 0; b < 4; b++)
            if (((v >> b) & 1) && ((n + b) >> 6) < nwords) flipb(out, n + b);
    }
    return n;
}

/* mtgp-calc-jump.hpp:34-58 (polytostring). */
int orc_gf2_to_hex(const uint64_t *p, int degree, char *out, int cap) {
    static const char digits[] = "0123456789abcdef";
    int nd = degree / 4 + 1;
    if (nd + 1 > cap) return -1;
    for (int k = 0; k < nd; k++) {
        int v = 0;
        for (int b = 0; b < 4; b++) {
            int i = 4 * k + b;
            if (i <= degree && getb(p, i)) v |= 1 << b;
        }
        out[k] = digits[v];
    }
    out[nd] = '\0';
    return nd;
}
