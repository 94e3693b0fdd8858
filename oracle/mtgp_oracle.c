/*
 * mtgp_oracle.c -- CPU restatement of the MTGP reference (test oracle).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg; never by the product library.
 *
 * Every function follows the cited lines of MersenneTwister-Lab/MTGP v1.1.2.
 * The state is kept exactly as the reference keeps it (a power-of-two ring of
 * large_size words and an index of the newest word), so whole rings can be
 * compared, not only the live window.
 */
#include "mtgp_oracle.h"

#include <ctype.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc32 {
    mtgp32_params_fast_t p;
    int size, lsize, lmask, idx;
    uint32_t *a;
};

struct orc64 {
    mtgp64_params_fast_t p;
    int size, lsize, lmask, idx;
    uint64_t *a;
};

/* size = mexp/w + 1 and the smallest power of two above it
 * (mtgp32-fast.c:36-58, mtgp64-fast.c:36-58). */
static int ring_size(int size) {
    int x = 1;
    while (x <= size) x <<= 1;
    return x;
}

/* ======================================================================= */
/* 32-bit                                                                  */
/* ======================================================================= */

static orc32_t *orc32_alloc(const mtgp32_params_fast_t *p) {
    orc32_t *o = (orc32_t *)calloc(1, sizeof(orc32_t));
    if (!o) return NULL;
    o->p = *p;
    o->size = p->mexp / 32 + 1;
    o->lsize = ring_size(o->size);
    o->lmask = o->lsize - 1;
    o->a = (uint32_t *)calloc((size_t)o->lsize, sizeof(uint32_t));
    if (!o->a) { free(o); return NULL; }
    o->idx = o->size - 1;
    return o;
}

/* mtgp32-fast.c:119-137 (mtgp32_init_state). */
static void seed32(uint32_t *a, const mtgp32_params_fast_t *p, uint32_t seed) {
    int size = p->mexp / 32 + 1;
    uint32_t hidden = p->tbl[4] ^ (p->tbl[8] << 16);
    uint32_t fillb = hidden;
    fillb += fillb >> 16;
    fillb += fillb >> 8;
    uint32_t word = (fillb & 0xffu) * 0x01010101u;
    for (int i = 0; i < size; i++) a[i] = word;
    a[0] = seed;
    a[1] = hidden;
    for (int i = 1; i < size; i++)
        a[i] ^= 1812433253u * (a[i - 1] ^ (a[i - 1] >> 30)) + (uint32_t)i;
}

orc32_t *orc32_new_seed(const mtgp32_params_fast_t *p, uint32_t seed) {
    orc32_t *o = orc32_alloc(p);           /* mtgp32-fast.c:94-104 */
    if (!o) return NULL;
    seed32(o->a, p, seed);
    return o;
}

/* mtgp32-fast.c:151-235 (init_by_array) and :250-334 (init_by_str); the two
 * differ only in where the key comes from.  Key bytes of the string form are
 * taken as signed char, as the reference behaves on x86-64. */
static void keyed32(orc32_t *o, const uint32_t *key, const char *skey,
                    int len) {
    const int size = o->size;
    uint32_t *a = o->a;
    int lag = size >= 623 ? 11 : size >= 68 ? 7 : size >= 39 ? 5 : 3;
    int mid = (size - lag) / 2;
    uint32_t hidden = o->p.tbl[4] ^ (o->p.tbl[8] << 16);
    uint32_t fillb = hidden;
    fillb += fillb >> 16;
    fillb += fillb >> 8;
    uint32_t word = (fillb & 0xffu) * 0x01010101u;
    for (int k = 0; k < size; k++) a[k] = word;
    a[0] = hidden;
    int total = (len + 1 > size) ? len + 1 : size;
    uint32_t r = a[0] ^ a[mid] ^ a[size - 1];
    r = (r ^ (r >> 27)) * 1664525u;
    a[mid] += r;
    r += (uint32_t)len;
    a[(mid + lag) % size] += r;
    a[0] = r;
    total--;
    int i = 1, j = 0;
    for (; j < total && j < len; j++) {
        uint32_t t = a[i] ^ a[(i + mid) % size] ^ a[(i + size - 1) % size];
        t = (t ^ (t >> 27)) * 1664525u;
        a[(i + mid) % size] += t;
        uint32_t k = key ? key[j] : (uint32_t)(int)(signed char)skey[j];
        t += k + (uint32_t)i;
        a[(i + mid + lag) % size] += t;
        a[i] = t;
        i = (i + 1) % size;
    }
    for (; j < total; j++) {
        uint32_t t = a[i] ^ a[(i + mid) % size] ^ a[(i + size - 1) % size];
        t = (t ^ (t >> 27)) * 1664525u;
        a[(i + mid) % size] += t;
        t += (uint32_t)i;
        a[(i + mid + lag) % size] += t;
        a[i] = t;
        i = (i + 1) % size;
    }
    for (j = 0; j < size; j++) {
        uint32_t t = a[i] + a[(i + mid) % size] + a[(i + size - 1) % size];
        t = (t ^ (t >> 27)) * 1566083941u;
        a[(i + mid) % size] ^= t;
        t -= (uint32_t)i;
        a[(i + mid + lag) % size] ^= t;
        a[i] = t;
        i = (i + 1) % size;
    }
    if (a[size - 1] == 0) a[size - 1] = 0x4d544750u;
}

orc32_t *orc32_new_array(const mtgp32_params_fast_t *p, const uint32_t *k,
                         int len) {
    orc32_t *o = orc32_alloc(p);
    if (!o) return NULL;
    keyed32(o, k, NULL, len);
    return o;
}

orc32_t *orc32_new_str(const mtgp32_params_fast_t *p, const char *s) {
    orc32_t *o = orc32_alloc(p);
    if (!o) return NULL;
    keyed32(o, NULL, s, (int)strlen(s));
    return o;
}

orc32_t *orc32_clone(const orc32_t *src) {
    orc32_t *o = orc32_alloc(&src->p);
    if (!o) return NULL;
    memcpy(o->a, src->a, sizeof(uint32_t) * (size_t)src->lsize);
    o->idx = src->idx;
    return o;
}

void orc32_delete(orc32_t *o) {
    if (!o) return;
    free(o->a);
    free(o);
}

int orc32_size(const orc32_t *o) { return o->size; }

/* mtgp32-fast.h:149-159 (do_recursion) + :165-183 (next_state): returns the
 * new word now stored at the newest ring position. */
static inline uint32_t step32(orc32_t *o) {
    const int n = o->size, L = o->lsize, m = o->lmask;
    o->idx = (o->idx + 1) & m;
    const int i = o->idx;
    uint32_t x1 = o->a[(i - n + L) & m];
    uint32_t x2 = o->a[(i - n + L + 1) & m];
    uint32_t y = o->a[(i + o->p.pos - n + L) & m];
    uint32_t x = (x1 & o->p.mask) ^ x2;
    x ^= x << o->p.sh1;
    y = x ^ (y >> o->p.sh2);
    uint32_t r = y ^ o->p.tbl[y & 0x0f];
    o->a[i] = r;
    return r;
}

/* Tempering helper word for the newest output (mtgp32-fast.h:263-266). */
static inline uint32_t fold32(const orc32_t *o) {
    uint32_t t = o->a[(o->idx + o->p.pos - 1 - o->size + o->lsize) & o->lmask];
    t ^= t >> 16;
    t ^= t >> 8;
    return t & 0x0f;
}

static inline float bits_to_float(uint32_t u) {
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}

void orc32_fill(orc32_t *o, int kind, void *out, size_t n) {
    uint32_t *u = (uint32_t *)out;
    float *f = (float *)out;
    for (size_t k = 0; k < n; k++) {
        uint32_t r = step32(o);
        uint32_t t = fold32(o);
        switch (kind) {
        case MTGP_KIND_UINT:          /* mtgp32-fast.h:192-198, 252-267 */
            u[k] = r ^ o->p.tmp_tbl[t];
            break;
        case MTGP_KIND_CLOSE1_OPEN2:  /* :207-218, 278-293 */
            f[k] = bits_to_float((r >> 9) ^ o->p.flt_tmp_tbl[t]);
            break;
        case MTGP_KIND_CLOSE_OPEN:    /* :304-306 */
            f[k] = bits_to_float((r >> 9) ^ o->p.flt_tmp_tbl[t]) - 1.0F;
            break;
        case MTGP_KIND_OPEN_CLOSE:    /* :317-319 */
            f[k] = 2.0F - bits_to_float((r >> 9) ^ o->p.flt_tmp_tbl[t]);
            break;
        default:                      /* :228-239, 330-346 */
            f[k] = bits_to_float(((r >> 9) ^ o->p.flt_tmp_tbl[t]) | 1u) - 1.0F;
            break;
        }
    }
}

void orc32_skip(orc32_t *o, uint64_t n) {
    for (uint64_t k = 0; k < n; k++) step32(o);
}

/* mtgp32-fast-jump.c:29-44 (add): XOR src's ring into dst's, aligned so that
 * the newest words coincide. */
static void add32(orc32_t *dst, const orc32_t *src) {
    const int L = src->lsize;
    const int shift = (src->idx - dst->idx + L) % L;
    for (int k = 0; k < L; k++) dst->a[k] ^= src->a[(k + shift) % L];
}

/* mtgp32-fast-jump.c:51-79: for each coefficient c_i, LSB first, add the
 * state when c_i is set, then step the state once. */
static void jump32_bits(orc32_t *o, const uint8_t *coef, int ncoef) {
    orc32_t *acc = orc32_alloc(&o->p);
    memset(acc->a, 0, sizeof(uint32_t) * (size_t)acc->lsize);
    acc->idx = acc->lsize - 1;
    for (int i = 0; i < ncoef; i++) {
        if (coef[i]) add32(acc, o);
        step32(o);
    }
    memcpy(o->a, acc->a, sizeof(uint32_t) * (size_t)o->lsize);
    o->idx = acc->idx;
    orc32_delete(acc);
}

static int hex_coeffs(const char *hex, uint8_t **out) {
    size_t len = strlen(hex);
    uint8_t *c = (uint8_t *)malloc(len * 4 + 1);
    if (!c) return -1;
    for (size_t k = 0; k < len; k++) {
        int ch = (unsigned char)hex[k];
        if (!isxdigit(ch)) { free(c); return -1; }
        ch = tolower(ch);
        int v = (ch >= 'a') ? ch - 'a' + 10 : ch - '0';
        for (int b = 0; b < 4; b++) c[4 * k + b] = (uint8_t)((v >> b) & 1);
    }
    *out = c;
    return (int)(len * 4);
}

int orc32_fast_jump(orc32_t *o, const char *hex) {
    uint8_t *c = NULL;
    int nc = hex_coeffs(hex, &c);
    if (nc < 0) return MTGP_ERR_BAD_JUMP;
    jump32_bits(o, c, nc);
    free(c);
    return 0;
}

void orc32_jump_words(orc32_t *o, const uint32_t *w, int nwords) {
    uint8_t *c = (uint8_t *)malloc((size_t)nwords * 32 + 1);
    for (int i = 0; i < nwords * 32; i++) c[i] = (uint8_t)((w[i / 32] >> (i % 32)) & 1);
    jump32_bits(o, c, nwords * 32);
    free(c);
}

/* Live window, oldest first: ring[(idx - size + 1 + k) & mask]. */
void orc32_get_window(const orc32_t *o, uint32_t *win) {
    for (int k = 0; k < o->size; k++)
        win[k] = o->a[(o->idx - o->size + 1 + k + o->lsize) & o->lmask];
}

void orc32_set_window(orc32_t *o, const uint32_t *win) {
    memset(o->a, 0, sizeof(uint32_t) * (size_t)o->lsize);
    for (int k = 0; k < o->size; k++) o->a[k] = win[k];
    o->idx = o->size - 1;
}

int orc32_get_ring(const orc32_t *o, uint32_t *ring) {
    memcpy(ring, o->a, sizeof(uint32_t) * (size_t)o->lsize);
    return o->idx;
}

/* ======================================================================= */
/* 64-bit                                                                  */
/* ======================================================================= */

static orc64_t *orc64_alloc(const mtgp64_params_fast_t *p) {
    orc64_t *o = (orc64_t *)calloc(1, sizeof(orc64_t));
    if (!o) return NULL;
    o->p = *p;
    o->size = p->mexp / 64 + 1;
    o->lsize = ring_size(o->size);
    o->lmask = o->lsize - 1;
    o->a = (uint64_t *)calloc((size_t)o->lsize, sizeof(uint64_t));
    if (!o->a) { free(o); return NULL; }
    o->idx = o->size - 1;
    return o;
}

/* mtgp64-fast.c:124-142 (mtgp64_init_state). */
static void seed64(uint64_t *a, const mtgp64_params_fast_t *p, uint64_t seed) {
    int size = p->mexp / 64 + 1;
    uint64_t hidden = p->tbl[4] ^ (p->tbl[8] << 16);
    uint64_t fillb = hidden >> 32;
    fillb += fillb >> 16;
    fillb += fillb >> 8;
    uint64_t word = (fillb & 0xffu) * UINT64_C(0x0101010101010101);
    for (int i = 0; i < size; i++) a[i] = word;
    a[0] = seed;
    a[1] = hidden;
    for (int i = 1; i < size; i++)
        a[i] ^= UINT64_C(6364136223846793005) * (a[i - 1] ^ (a[i - 1] >> 62))
                + (uint64_t)i;
}

orc64_t *orc64_new_seed(const mtgp64_params_fast_t *p, uint64_t seed) {
    orc64_t *o = orc64_alloc(p);           /* mtgp64-fast.c:99-109 */
    if (!o) return NULL;
    seed64(o->a, p, seed);
    return o;
}

/* mtgp64-fast.c:156-239 (init_by_array) and :255-339 (init_by_str). */
static void keyed64(orc64_t *o, const uint64_t *key, const char *skey,
                    int len) {
    const int size = o->size;
    uint64_t *a = o->a;
    int lag = size >= 623 ? 11 : size >= 68 ? 7 : size >= 39 ? 5 : 3;
    int mid = (size - lag) / 2;
    uint64_t hidden = o->p.tbl[4] ^ (o->p.tbl[8] << 16);
    uint64_t fillb = hidden >> 32;
    fillb += fillb >> 16;
    fillb += fillb >> 8;
    uint64_t word = (fillb & 0xffu) * UINT64_C(0x0101010101010101);
    for (int k = 0; k < size; k++) a[k] = word;
    a[0] = hidden;
    int total = (len + 1 > size) ? len + 1 : size;
    const uint64_t m1 = UINT64_C(2173292883993), m2 = UINT64_C(58885565329898161);
    uint64_t r = a[0] ^ a[mid] ^ a[size - 1];
    r = (r ^ (r >> 59)) * m1;
    a[mid] += r;
    r += (uint64_t)len;
    a[(mid + lag) % size] += r;
    a[0] = r;
    total--;
    int i = 1, j = 0;
    for (; j < total && j < len; j++) {
        uint64_t t = a[i] ^ a[(i + mid) % size] ^ a[(i + size - 1) % size];
        t = (t ^ (t >> 59)) * m1;
        a[(i + mid) % size] += t;
        if (key)
            t += key[j] + (uint64_t)i;
        else
            t += (uint64_t)(int64_t)((int)(signed char)skey[j] + i);
        a[(i + mid + lag) % size] += t;
        a[i] = t;
        i = (i + 1) % size;
    }
    for (; j < total; j++) {
        uint64_t t = a[i] ^ a[(i + mid) % size] ^ a[(i + size - 1) % size];
        t = (t ^ (t >> 59)) * m1;
        a[(i + mid) % size] += t;
        t += (uint64_t)i;
        a[(i + mid + lag) % size] += t;
        a[i] = t;
        i = (i + 1) % size;
    }
    for (j = 0; j < size; j++) {
        uint64_t t = a[i] + a[(i + mid) % size] + a[(i + size - 1) % size];
        t = (t ^ (t >> 59)) * m2;
        a[(i + mid) % size] ^= t;
        t -= (uint64_t)i;
        a[(i + mid + lag) % size] ^= t;
        a[i] = t;
        i = (i + 1) % size;
    }
    if (a[size - 1] == 0) a[size - 1] = 0x4d544750u;
}

orc64_t *orc64_new_array(const mtgp64_params_fast_t *p, const uint64_t *k,
                         int len) {
    orc64_t *o = orc64_alloc(p);
    if (!o) return NULL;
    keyed64(o, k, NULL, len);
    return o;
}

orc64_t *orc64_new_str(const mtgp64_params_fast_t *p, const char *s) {
    orc64_t *o = orc64_alloc(p);
    if (!o) return NULL;
    keyed64(o, NULL, s, (int)strlen(s));
    return o;
}

orc64_t *orc64_clone(const orc64_t *src) {
    orc64_t *o = orc64_alloc(&src->p);
    if (!o) return NULL;
    memcpy(o->a, src->a, sizeof(uint64_t) * (size_t)src->lsize);
    o->idx = src->idx;
    return o;
}

void orc64_delete(orc64_t *o) {
    if (!o) return;
    free(o->a);
    free(o);
}

int orc64_size(const orc64_t *o) { return o->size; }

/* mtgp64-fast.h:148-169 (do_recursion: the two 32-bit halves are shifted
 * separately and cross over) + :175-193 (next_state). */
static inline uint64_t step64(orc64_t *o) {
    const int n = o->size, L = o->lsize, m = o->lmask;
    o->idx = (o->idx + 1) & m;
    const int i = o->idx;
    uint64_t x1 = o->a[(i - n + L) & m];
    uint64_t x2 = o->a[(i - n + L + 1) & m];
    uint64_t y = o->a[(i + o->p.pos - n + L) & m];
    uint64_t x = (x1 & o->p.mask) ^ x2;
    uint32_t xh = (uint32_t)(x >> 32), xl = (uint32_t)x;
    uint32_t yh = (uint32_t)(y >> 32), yl = (uint32_t)y;
    xh ^= xh << o->p.sh1;
    xl ^= xl << o->p.sh1;
    yh = xl ^ (yh >> o->p.sh2);
    yl = xh ^ (yl >> o->p.sh2);
    uint64_t r = ((uint64_t)yh << 32) | yl;
    r ^= o->p.tbl[yl & 0x0f];
    o->a[i] = r;
    return r;
}

static inline uint32_t fold64(const orc64_t *o) {
    uint64_t t = o->a[(o->idx + o->p.pos - 1 - o->size + o->lsize) & o->lmask];
    t ^= t >> 16;
    t ^= t >> 8;
    return (uint32_t)(t & 0x0f);
}

static inline double bits_to_double(uint64_t u) {
    double d;
    memcpy(&d, &u, sizeof d);
    return d;
}

void orc64_fill(orc64_t *o, int kind, void *out, size_t n) {
    uint64_t *u = (uint64_t *)out;
    double *d = (double *)out;
    for (size_t k = 0; k < n; k++) {
        uint64_t r = step64(o);
        uint32_t t = fold64(o);
        switch (kind) {
        case MTGP_KIND_UINT:          /* mtgp64-fast.h:202-208, 262-277 */
            u[k] = r ^ o->p.tmp_tbl[t];
            break;
        case MTGP_KIND_CLOSE1_OPEN2:  /* :217-228, 288-303 */
            d[k] = bits_to_double((r >> 12) ^ o->p.dbl_tmp_tbl[t]);
            break;
        case MTGP_KIND_CLOSE_OPEN:    /* :314-316 */
            d[k] = bits_to_double((r >> 12) ^ o->p.dbl_tmp_tbl[t]) - 1.0;
            break;
        case MTGP_KIND_OPEN_CLOSE:    /* :327-329 */
            d[k] = 2.0 - bits_to_double((r >> 12) ^ o->p.dbl_tmp_tbl[t]);
            break;
        default:  /* :238-249, 340-356: the |1 is applied BEFORE the XOR */
            d[k] = bits_to_double(((r >> 12) | 1u) ^ o->p.dbl_tmp_tbl[t]) - 1.0;
            break;
        }
    }
}

void orc64_skip(orc64_t *o, uint64_t n) {
    for (uint64_t k = 0; k < n; k++) step64(o);
}

static void add64(orc64_t *dst, const orc64_t *src) {
    const int L = src->lsize;
    const int shift = (src->idx - dst->idx + L) % L;
    for (int k = 0; k < L; k++) dst->a[k] ^= src->a[(k + shift) % L];
}

/* mtgp64-fast-jump.c:51-79. */
static void jump64_bits(orc64_t *o, const uint8_t *coef, int ncoef) {
    orc64_t *acc = orc64_alloc(&o->p);
    memset(acc->a, 0, sizeof(uint64_t) * (size_t)acc->lsize);
    acc->idx = acc->lsize - 1;
    for (int i = 0; i < ncoef; i++) {
        if (coef[i]) add64(acc, o);
        step64(o);
    }
    memcpy(o->a, acc->a, sizeof(uint64_t) * (size_t)o->lsize);
    o->idx = acc->idx;
    orc64_delete(acc);
}

int orc64_fast_jump(orc64_t *o, const char *hex) {
    uint8_t *c = NULL;
    int nc = hex_coeffs(hex, &c);
    if (nc < 0) return MTGP_ERR_BAD_JUMP;
    jump64_bits(o, c, nc);
    free(c);
    return 0;
}

void orc64_jump_words(orc64_t *o, const uint32_t *w, int nwords) {
    uint8_t *c = (uint8_t *)malloc((size_t)nwords * 32 + 1);
    for (int i = 0; i < nwords * 32; i++) c[i] = (uint8_t)((w[i / 32] >> (i % 32)) & 1);
    jump64_bits(o, c, nwords * 32);
    free(c);
}

void orc64_get_window(const orc64_t *o, uint64_t *win) {
    for (int k = 0; k < o->size; k++)
        win[k] = o->a[(o->idx - o->size + 1 + k + o->lsize) & o->lmask];
}

void orc64_set_window(orc64_t *o, const uint64_t *win) {
    memset(o->a, 0, sizeof(uint64_t) * (size_t)o->lsize);
    for (int k = 0; k < o->size; k++) o->a[k] = win[k];
    o->idx = o->size - 1;
}

int orc64_get_ring(const orc64_t *o, uint64_t *ring) {
    memcpy(ring, o->a, sizeof(uint64_t) * (size_t)o->lsize);
    return o->idx;
}

/* ======================================================================= */
/* Many generators (CPU baseline: OpenMP over generators)                  */
/* ======================================================================= */

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc32_seed_windows(const mtgp32_params_fast_t *params,
                        const int *param_idx, const uint32_t *seeds, int ngen,
                        uint32_t *windows) {
    for (int g = 0; g < ngen; g++) {
        const mtgp32_params_fast_t *p = &params[param_idx ? param_idx[g] : g];
        int size = p->mexp / 32 + 1;
        seed32(windows + (size_t)g * size, p, seeds[g]);
    }
}

void orc64_seed_windows(const mtgp64_params_fast_t *params,
                        const int *param_idx, const uint64_t *seeds, int ngen,
                        uint64_t *windows) {
    for (int g = 0; g < ngen; g++) {
        const mtgp64_params_fast_t *p = &params[param_idx ? param_idx[g] : g];
        int size = p->mexp / 64 + 1;
        seed64(windows + (size_t)g * size, p, seeds[g]);
    }
}

void orc32_multi_fill(const mtgp32_params_fast_t *params, int nparams,
                      const int *param_idx, uint32_t *windows, int ngen,
                      const uint64_t *counts, const int *kinds,
                      const uint64_t *offsets, void *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#else
    (void)nthreads;
#endif
    for (int g = 0; g < ngen; g++) {
        const mtgp32_params_fast_t *p = &params[param_idx ? param_idx[g] : g % nparams];
        orc32_t *o = orc32_alloc(p);
        int size = o->size;
        orc32_set_window(o, windows + (size_t)g * size);
        orc32_fill(o, kinds ? kinds[g] : 0, (char *)out + offsets[g], counts[g]);
        orc32_get_window(o, windows + (size_t)g * size);
        orc32_delete(o);
    }
}

void orc64_multi_fill(const mtgp64_params_fast_t *params, int nparams,
                      const int *param_idx, uint64_t *windows, int ngen,
                      const uint64_t *counts, const int *kinds,
                      const uint64_t *offsets, void *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#else
    (void)nthreads;
#endif
    for (int g = 0; g < ngen; g++) {
        const mtgp64_params_fast_t *p = &params[param_idx ? param_idx[g] : g % nparams];
        orc64_t *o = orc64_alloc(p);
        int size = o->size;
        orc64_set_window(o, windows + (size_t)g * size);
        orc64_fill(o, kinds ? kinds[g] : 0, (char *)out + offsets[g], counts[g]);
        orc64_get_window(o, windows + (size_t)g * size);
        orc64_delete(o);
    }
}
