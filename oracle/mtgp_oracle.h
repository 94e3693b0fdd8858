/*
 * mtgp_oracle.h -- CPU restatement of the MTGP reference algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU path is checked
 * against; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  The product library never links or calls it.
 *
 * It restates, function by function, the reference's portable C code
 * (MersenneTwister-Lab/MTGP v1.1.2: mtgp32-fast.{h,c}, mtgp64-fast.{h,c},
 * mtgp32-fast-jump.c, mtgp64-fast-jump.c); each function cites the lines it
 * follows.  The restatement itself is pinned against golden vectors produced
 * by the reference compiled from its own sources (tests/golden/), and against
 * the reference library directly where it can be built (oracle/_ref).
 *
 * GF(2)[x] helpers (Berlekamp-Massey, X^e mod chi) restate the published
 * algorithms that the reference takes from NTL (MinPolySeq, PowerXMod; used
 * in mtgp32-calc-poly.cpp:36-45 and mtgp-calc-jump.hpp:135-162).  They are
 * deliberately simple, bit-serial code.
 */
#ifndef MTGP_ORACLE_H
#define MTGP_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/mtgp_gpu.h"

#if defined(__cplusplus)
extern "C" {
#endif

typedef struct orc32 orc32_t;
typedef struct orc64 orc64_t;

/* ---- 32-bit ---- */
orc32_t *orc32_new_seed(const mtgp32_params_fast_t *p, uint32_t seed);
orc32_t *orc32_new_array(const mtgp32_params_fast_t *p, const uint32_t *a,
                         int len);
orc32_t *orc32_new_str(const mtgp32_params_fast_t *p, const char *s);
orc32_t *orc32_clone(const orc32_t *o);
void orc32_delete(orc32_t *o);
int orc32_size(const orc32_t *o);
/* kind: MTGP_KIND_*; out holds n uint32 (kind 0) or n float. */
void orc32_fill(orc32_t *o, int kind, void *out, size_t n);
void orc32_skip(orc32_t *o, uint64_t n);
/* 0 on success, MTGP_ERR_BAD_JUMP on a non-hex character. */
int orc32_fast_jump(orc32_t *o, const char *hex);
void orc32_jump_words(orc32_t *o, const uint32_t *w, int nwords);
void orc32_get_window(const orc32_t *o, uint32_t *win);
void orc32_set_window(orc32_t *o, const uint32_t *win);
/* Full ring (large_size words) and idx, for whole-array comparisons. */
int orc32_get_ring(const orc32_t *o, uint32_t *ring);

/* ---- 64-bit ---- */
orc64_t *orc64_new_seed(const mtgp64_params_fast_t *p, uint64_t seed);
orc64_t *orc64_new_array(const mtgp64_params_fast_t *p, const uint64_t *a,
                         int len);
orc64_t *orc64_new_str(const mtgp64_params_fast_t *p, const char *s);
orc64_t *orc64_clone(const orc64_t *o);
void orc64_delete(orc64_t *o);
int orc64_size(const orc64_t *o);
void orc64_fill(orc64_t *o, int kind, void *out, size_t n);
void orc64_skip(orc64_t *o, uint64_t n);
int orc64_fast_jump(orc64_t *o, const char *hex);
void orc64_jump_words(orc64_t *o, const uint32_t *w, int nwords);
void orc64_get_window(const orc64_t *o, uint64_t *win);
void orc64_set_window(orc64_t *o, const uint64_t *win);
int orc64_get_ring(const orc64_t *o, uint64_t *ring);

/* ---- many generators, OpenMP over generators (CPU baseline) ----
 * Generator g is (params[g], windows[g*size .. (g+1)*size)) and writes
 * counts[g] values of kinds[g] at byte offset offsets[g] of out.
 * windows are updated in place.  nthreads <= 0: OpenMP default. */
void orc32_multi_fill(const mtgp32_params_fast_t *params, int nparams,
                      const int *param_idx, uint32_t *windows, int ngen,
                      const uint64_t *counts, const int *kinds,
                      const uint64_t *offsets, void *out, int nthreads);
void orc64_multi_fill(const mtgp64_params_fast_t *params, int nparams,
                      const int *param_idx, uint64_t *windows, int ngen,
                      const uint64_t *counts, const int *kinds,
                      const uint64_t *offsets, void *out, int nthreads);
int orc_max_threads(void);

/* Windows (oldest first) of ngen generators seeded with seeds[g]. */
void orc32_seed_windows(const mtgp32_params_fast_t *params,
                        const int *param_idx, const uint32_t *seeds, int ngen,
                        uint32_t *windows);
void orc64_seed_windows(const mtgp64_params_fast_t *params,
                        const int *param_idx, const uint64_t *seeds, int ngen,
                        uint64_t *windows);

/* ---- GF(2)[x] (polynomials are uint64 words, bit i of the whole array is
 * the coefficient of X^i) ---- */
/* Minimal polynomial of bits[0..n) (one bit per byte) by Berlekamp-Massey;
 * writes coefficients into out (nwords words), returns the degree. */
int orc_gf2_minpoly(const uint8_t *bits, int n, uint64_t *out, int nwords);
/* out = X^e mod m; e is a little-endian array of ewords uint32 words;
 * m has degree dm.  out has (dm + 63) / 64 words. */
void orc_gf2_powxmod(const uint32_t *e, int ewords, const uint64_t *m, int dm,
                     uint64_t *out);
/* out = a * b mod m (a, b of degree < dm). */
void orc_gf2_mulmod(const uint64_t *a, const uint64_t *b, const uint64_t *m,
                    int dm, uint64_t *out);
/* Parse / print the reference's hex polynomial form (mtgp-calc-jump.hpp:
 * 34-58, 98-126).  parse returns the number of coefficients read (4 per
 * digit) or -1 on a bad digit. */
int orc_gf2_from_hex(const char *hex, uint64_t *out, int nwords);
int orc_gf2_to_hex(const uint64_t *p, int degree, char *out, int cap);

#if defined(__cplusplus)
}
#endif
#endif
