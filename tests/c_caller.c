/*
 * c_caller.c -- a plain C caller of libmtgp_gb300.so (tests/test_c_caller.py).
 *
 * Built two ways:
 *   -DWITH_REF  the reference's own headers (mtgp32-fast.h, mtgp64-fast.h) are
 *               included first and its parameter table (mtgp32-param-fast.c,
 *               compiled from the reference tree) is linked in: the library's
 *               header must then take the reference's struct definitions,
 *               and the reference's table must be usable as the ABI's
 *               parameter argument unchanged (mtgp32-fast.h:47-88).
 *   otherwise   mtgp_gpu.h alone, with its own definitions of the same types;
 *               the parameter set is read from a file of raw structs.
 *
 * Modes (argv[1]):
 *   abi FILE   calls that need no GPU: version, tuning, argument errors;
 *              prints "abi ok"
 *   gen FILE   (GPU) generator from parameter set 0 (FILE: raw
 *              mtgp32_params_fast_t structs, ignored with -DWITH_REF), seed
 *              1234: 1000 uint32 and 1000 float [0,1) into device memory,
 *              printed one value per line as hex words
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef WITH_REF
#include "mtgp32-fast.h"
#include "mtgp64-fast.h"
#endif
#include "mtgp_gpu.h"

/* The CUDA runtime calls this caller needs (from libcudart). */
int cudaMalloc(void **p, size_t n);
int cudaMemcpy(void *dst, const void *src, size_t n, int kind);
int cudaFree(void *p);
int cudaDeviceSynchronize(void);

static int abi_checks(const mtgp32_params_fast_t *p) {
    if (sizeof(mtgp32_params_fast_t) != 236 || sizeof(mtgp64_params_fast_t) != 432) {
        printf("struct sizes %zu %zu\n", sizeof(mtgp32_params_fast_t),
               sizeof(mtgp64_params_fast_t));
        return 1;
    }
    if (p->mexp != 11213) {
        printf("parameter set mexp %d\n", p->mexp);
        return 1;
    }
#define CHECK(c)                                          \
    do {                                                  \
        if (!(c)) {                                       \
            printf("failed at line %d: %s\n", __LINE__, #c); \
            return 1;                                     \
        }                                                 \
    } while (0)
    CHECK(mtgp_gpu_version() && strstr(mtgp_gpu_version(), "sm_103a"));
    CHECK(mtgp_gpu_set_tuning("core", 2) == MTGP_OK);
    CHECK(mtgp_gpu_set_tuning("core", 3) == MTGP_ERR_INVALID);
    CHECK(mtgp32_gpu_pool_set_tuning(NULL, "core", 2) == MTGP_ERR_INVALID);
    CHECK(mtgp32_gpu_init(NULL, p, 1) == MTGP_ERR_INVALID);
    CHECK(mtgp32_gpu_fill_uint32(NULL, NULL, 10, NULL) == MTGP_ERR_INVALID);
    CHECK(mtgp_gpu_last_error() != NULL);
#undef CHECK
    printf("abi ok\n");
    return 0;
}

static int gen(const mtgp32_params_fast_t *p) {
    mtgp32_gpu_t *g = NULL;
    void *d = NULL;
    uint32_t host[2000];
    int rc = mtgp32_gpu_init(&g, p, 1234);
    if (rc) {
        printf("init: %d %s\n", rc, mtgp_gpu_last_error());
        return 1;
    }
    if (cudaMalloc(&d, sizeof host)) return 1;
    rc = mtgp32_gpu_fill_uint32(g, (uint32_t *)d, 1000, NULL);
    if (!rc) rc = mtgp32_gpu_fill_close_open(g, (float *)d + 1000, 1000, NULL);
    if (rc) {
        printf("fill: %d %s\n", rc, mtgp_gpu_last_error());
        return 1;
    }
    if (cudaDeviceSynchronize() || cudaMemcpy(host, d, sizeof host, 2 /* DeviceToHost */))
        return 1;
    for (int k = 0; k < 2000; k++) printf("%08x\n", (unsigned)host[k]);
    cudaFree(d);
    mtgp32_gpu_free(g);
    return 0;
}

int main(int argc, char **argv) {
    mtgp32_params_fast_t p;
#ifdef WITH_REF
    p = mtgp32_params_fast_11213[0];
#else
    FILE *f = argc >= 3 ? fopen(argv[2], "rb") : NULL;
    if (!f || fread(&p, sizeof p, 1, f) != 1) {
        printf("cannot read the parameter file\n");
        return 1;
    }
    fclose(f);
#endif
    if (argc >= 2 && !strcmp(argv[1], "gen")) return gen(&p);
    return abi_checks(&p);
}
