/*
 * ref_shim.c -- thin driver around the reference library itself.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile, target `ref`)
 * together with the unmodified reference sources read in place from the
 * reference tree into oracle/_ref/libmtgpref.so.  The reference's genrand_*
 * are static inline functions in its headers, so they cannot be called
 * through a shared library directly; this file exposes them as plain loops
 * (fill = n successive genrand_* calls), plus the reference's fast_jump and
 * its parameter / jump tables, for the golden-vector generator and the
 * CPU baseline ("reference" kind).  Nothing here re-implements the algorithm.
 */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mtgp32-fast.h"
#include "mtgp64-fast.h"
#include "mtgp32-fast-jump.h"
#include "mtgp64-fast-jump.h"
#include "mtgp32-jump-string.h"
#include "mtgp64-jump-string.h"
#define MTGP32_CHAR11213_H
#include "cuda-sample/mtgp32-char11213.h"

extern mtgp32_params_fast_t mtgp32dc_params_fast_11213[];
extern mtgp64_params_fast_t mtgp64dc_params_fast_11213[];          /* OpenCL */
extern mtgp64_params_fast_t mtgp64dc_cuda_params_fast_11213[];     /* CUDA   */
extern const uint32_t mtgp32_jump_table[];
extern const uint32_t mtgp64_jump_table[];

/* ---- tables ---------------------------------------------------------- */
const void *ref_table(const char *name, int *count) {
    struct { const char *n; const void *p; int c; } t[] = {
        {"mtgp32_fast_11213", mtgp32_params_fast_11213, 128},
        {"mtgp32_fast_23209", mtgp32_params_fast_23209, 128},
        {"mtgp32_fast_44497", mtgp32_params_fast_44497, 128},
        {"mtgp32dc_fast_11213", mtgp32dc_params_fast_11213, 200},
        {"mtgp64_fast_23209", mtgp64_params_fast_23209, 128},
        {"mtgp64_fast_44497", mtgp64_params_fast_44497, 128},
        {"mtgp64_fast_110503", mtgp64_params_fast_110503, 128},
        {"mtgp64dc_fast_11213", mtgp64dc_params_fast_11213, 200},
        {"mtgp64dc_cuda_fast_11213", mtgp64dc_cuda_params_fast_11213, 200},
        {"mtgp32_jump_11213", mtgp32_jump_table, 6 * 351},
        {"mtgp64_jump_11213", mtgp64_jump_table, 6 * 351},
    };
    for (size_t k = 0; k < sizeof t / sizeof t[0]; k++)
        if (!strcmp(t[k].n, name)) { *count = t[k].c; return t[k].p; }
    *count = 0;
    return NULL;
}
const char *ref_jump_string32(void) { return mtgp32_jump_string; }
const char *ref_jump_string64(void) { return mtgp64_jump_string; }
const char *ref_char32_11213(void) { return CHAR32_11213; }
int ref_sizeof_params32(void) { return (int)sizeof(mtgp32_params_fast_t); }
int ref_sizeof_params64(void) { return (int)sizeof(mtgp64_params_fast_t); }

/* ---- 32-bit ---------------------------------------------------------- */
mtgp32_fast_t *ref32_new(const mtgp32_params_fast_t *p, int how, uint32_t seed,
                         uint32_t *arr, int len, char *str) {
    mtgp32_fast_t *m = (mtgp32_fast_t *)calloc(1, sizeof *m);
    int rc = how == 0 ? mtgp32_init(m, p, seed)
           : how == 1 ? mtgp32_init_by_array(m, p, arr, len)
                      : mtgp32_init_by_str(m, p, str);
    if (rc) { free(m); return NULL; }
    return m;
}
void ref32_delete(mtgp32_fast_t *m) { mtgp32_free(m); free(m); }

void ref32_fill(mtgp32_fast_t *m, int kind, void *out, size_t n) {
    uint32_t *u = (uint32_t *)out;
    float *f = (float *)out;
    size_t k;
    switch (kind) {
    case 0: for (k = 0; k < n; k++) u[k] = mtgp32_genrand_uint32(m); break;
    case 1: for (k = 0; k < n; k++) f[k] = mtgp32_genrand_close1_open2(m); break;
    case 2: for (k = 0; k < n; k++) f[k] = mtgp32_genrand_close_open(m); break;
    case 3: for (k = 0; k < n; k++) f[k] = mtgp32_genrand_open_close(m); break;
    default: for (k = 0; k < n; k++) f[k] = mtgp32_genrand_open_open(m); break;
    }
}
void ref32_fast_jump(mtgp32_fast_t *m, const char *hex) {
    mtgp32_fast_jump(m, hex);
}
int ref32_ring(const mtgp32_fast_t *m, uint32_t *ring) {
    memcpy(ring, m->status->array, sizeof(uint32_t) * m->status->large_size);
    return m->status->idx;
}
void ref32_print_idstring(const mtgp32_fast_t *m, char *out, int cap) {
    int n = snprintf(out, cap, "mtgp32:%d:", m->params.mexp);
    for (int i = 0; i < 20 && n + 2 < cap; i++)
        n += snprintf(out + n, cap - n, "%02x", (unsigned)m->params.poly_sha1[i]);
}

/* ---- 64-bit ---------------------------------------------------------- */
mtgp64_fast_t *ref64_new(const mtgp64_params_fast_t *p, int how, uint64_t seed,
                         uint64_t *arr, int len, char *str) {
    mtgp64_fast_t *m = (mtgp64_fast_t *)calloc(1, sizeof *m);
    int rc = how == 0 ? mtgp64_init(m, p, seed)
           : how == 1 ? mtgp64_init_by_array(m, p, arr, len)
                      : mtgp64_init_by_str(m, p, str);
    if (rc) { free(m); return NULL; }
    return m;
}
void ref64_delete(mtgp64_fast_t *m) { mtgp64_free(m); free(m); }

void ref64_fill(mtgp64_fast_t *m, int kind, void *out, size_t n) {
    uint64_t *u = (uint64_t *)out;
    double *d = (double *)out;
    size_t k;
    switch (kind) {
    case 0: for (k = 0; k < n; k++) u[k] = mtgp64_genrand_uint64(m); break;
    case 1: for (k = 0; k < n; k++) d[k] = mtgp64_genrand_close1_open2(m); break;
    case 2: for (k = 0; k < n; k++) d[k] = mtgp64_genrand_close_open(m); break;
    case 3: for (k = 0; k < n; k++) d[k] = mtgp64_genrand_open_close(m); break;
    default: for (k = 0; k < n; k++) d[k] = mtgp64_genrand_open_open(m); break;
    }
}
void ref64_fast_jump(mtgp64_fast_t *m, const char *hex) {
    mtgp64_fast_jump(m, hex);
}
int ref64_ring(const mtgp64_fast_t *m, uint64_t *ring) {
    memcpy(ring, m->status->array, sizeof(uint64_t) * m->status->large_size);
    return m->status->idx;
}

/* ---- many generators: OpenMP over generators (CPU baseline) ----------
 * Generator g: seed seeds[g] on params[pidx[g]], then counts[g] values of
 * kinds[g] written at byte offset offsets[g]. */
void ref32_multi_seed_fill(const mtgp32_params_fast_t *params, const int *pidx,
                           const uint32_t *seeds, int ngen,
                           const uint64_t *counts, const int *kinds,
                           const uint64_t *offsets, void *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int g = 0; g < ngen; g++) {
        mtgp32_fast_t m;
        mtgp32_init(&m, &params[pidx ? pidx[g] : g], seeds[g]);
        ref32_fill(&m, kinds ? kinds[g] : 0, (char *)out + offsets[g], counts[g]);
        mtgp32_free(&m);
    }
}
void ref64_multi_seed_fill(const mtgp64_params_fast_t *params, const int *pidx,
                           const uint64_t *seeds, int ngen,
                           const uint64_t *counts, const int *kinds,
                           const uint64_t *offsets, void *out, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int g = 0; g < ngen; g++) {
        mtgp64_fast_t m;
        mtgp64_init(&m, &params[pidx ? pidx[g] : g], seeds[g]);
        ref64_fill(&m, kinds ? kinds[g] : 0, (char *)out + offsets[g], counts[g]);
        mtgp64_free(&m);
    }
}
int ref_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
