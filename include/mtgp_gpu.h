/*
 * mtgp_gpu.h -- C ABI of the GB300 MTGP generator.
 *
 * Drop-in GPU replacement for the MTGP reference C API (MersenneTwister-Lab/MTGP,
 * v1.1.2).  Every entry point below names the reference function it replaces.
 * The generated sequences are bit-identical to the reference's
 * mtgp32-fast.c / mtgp64-fast.c for the same parameter set, seed and offset,
 * floats included.
 *
 * Conventions
 *   - Plain C types only: pointers, sizes, ints.  CUDA streams are passed as
 *     `void *` (a cudaStream_t; NULL = legacy default stream).
 *   - Every function returns an int status (MTGP_OK == 0, negative on error);
 *     no C++ exception crosses this boundary.  The reference returns -1 on
 *     allocation failure (mtgp32-fast.c:49-51) and asserts on malformed jump
 *     strings (mtgp32-fast-jump.c:62); here both are status codes.
 *     mtgp_gpu_last_error() returns a per-thread message for the last failure.
 *   - Output buffers are caller-owned DEVICE memory unless a name says _host.
 *   - A handle is single-owner, like the reference's mtgp32_fast_t: calls on one
 *     handle must not race; different handles are independent.
 *   - Fills are asynchronous on the given stream; the handle's device state is
 *     advanced in stream order, so successive fills on one stream continue the
 *     sequence exactly like successive genrand_* calls.
 *
 * The parameter and state structs have the reference's layout
 * (mtgp32-fast.h:47-88, mtgp64-fast.h:46-87), so the reference's parameter
 * tables (mtgp32-param-fast.c, mtgp64-param-fast.c, ...) link unchanged.  If a
 * translation unit also includes the reference's mtgp32-fast.h / mtgp64-fast.h,
 * include those first: this header then uses their definitions.
 */
#ifndef MTGP_GPU_H
#define MTGP_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__cplusplus)
extern "C" {
#endif

/* ---- reference-layout types (mtgp32-fast.h:47-88) ------------------------ */
#if !defined(MTGP32_FAST_H)
#define MTGP_GPU_DEFINES_MTGP32_TYPES 1
typedef struct MTGP32_PARAMS_FAST_T {
    int mexp;                   /* Mersenne exponent                       */
    int pos;                    /* pick-up position                        */
    int sh1;                    /* shift 1                                 */
    int sh2;                    /* shift 2                                 */
    uint32_t tbl[16];           /* recursion table                         */
    uint32_t tmp_tbl[16];       /* tempering table                         */
    uint32_t flt_tmp_tbl[16];   /* tempering + [1,2) float packing table   */
    uint32_t mask;              /* state-space mask of the oldest word     */
    unsigned char poly_sha1[21];
} mtgp32_params_fast_t;

typedef struct MTGP32_STATUS_FAST_T {
    int idx;
    int size;
    int large_size;
    int large_mask;
    uint32_t array[];
} mtgp32_status_fast_t;

typedef struct MTGP32_FAST_T {
    mtgp32_params_fast_t params;
    mtgp32_status_fast_t *status;
} mtgp32_fast_t;
#endif

/* ---- reference-layout types (mtgp64-fast.h:46-87) ------------------------ */
#if !defined(MTGP64_FAST_H)
#define MTGP_GPU_DEFINES_MTGP64_TYPES 1
typedef struct MTGP64_PARAMS_FAST_T {
    int mexp;
    int pos;
    int sh1;
    int sh2;
    uint64_t tbl[16];
    uint64_t tmp_tbl[16];
    uint64_t dbl_tmp_tbl[16];
    uint64_t mask;
    unsigned char poly_sha1[21];
} mtgp64_params_fast_t;

typedef struct MTGP64_STATUS_FAST_T {
    int idx;
    int size;
    int large_size;
    int large_mask;
    uint64_t array[];
} mtgp64_status_fast_t;

typedef struct MTGP64_FAST_T {
    mtgp64_params_fast_t params;
    mtgp64_status_fast_t *status;
} mtgp64_fast_t;
#endif

/* ---- status codes -------------------------------------------------------- */
#define MTGP_OK               0
#define MTGP_ERR_ALLOC      (-1)  /* host or device allocation failed (ref: -1)  */
#define MTGP_ERR_INVALID    (-2)  /* NULL handle/pointer, bad size or parameter  */
#define MTGP_ERR_UNSUPPORTED (-3) /* parameter set shape not supported          */
#define MTGP_ERR_BAD_JUMP   (-4)  /* malformed jump string / polynomial         */
#define MTGP_ERR_CUDA       (-5)  /* CUDA runtime error (message has details)   */
#define MTGP_ERR_TIMEOUT    (-6)  /* a bounded device-side wait gave up         */
#define MTGP_ERR_BUDGET     (-7)  /* request exceeds the device-memory budget   */
#define MTGP_ERR_BUSY       (-8)  /* no free slot; retry later                  */

/* Output kinds; the numbering is shared by all fill/batch entry points. */
#define MTGP_KIND_UINT       0   /* genrand_uint32 / genrand_uint64          */
#define MTGP_KIND_CLOSE1_OPEN2 1 /* [1,2)  genrand_close1_open2              */
#define MTGP_KIND_CLOSE_OPEN 2   /* [0,1)  genrand_close_open                */
#define MTGP_KIND_OPEN_CLOSE 3   /* (0,1]  genrand_open_close                */
#define MTGP_KIND_OPEN_OPEN  4   /* (0,1)  genrand_open_open                 */

/* Message describing the calling thread's last failed call ("" if none). */
const char *mtgp_gpu_last_error(void);
/* Library version string. */
const char *mtgp_gpu_version(void);

/* ========================================================================= */
/* Single generator (replaces mtgp32_fast_t usage)                            */
/* ========================================================================= */
typedef struct mtgp32_gpu mtgp32_gpu_t;
typedef struct mtgp64_gpu mtgp64_gpu_t;

/* Replaces mtgp32_init (mtgp32-fast.c:94-104) + mtgp32_init_state (:119-137).
 * Allocates the device-resident state and seeds it on the device with
 * the reference's exact arithmetic. */
int mtgp32_gpu_init(mtgp32_gpu_t **out, const mtgp32_params_fast_t *para,
                    uint32_t seed);
/* Replaces mtgp32_init_by_array (mtgp32-fast.c:151-235). */
int mtgp32_gpu_init_by_array(mtgp32_gpu_t **out,
                             const mtgp32_params_fast_t *para,
                             const uint32_t *array, int length);
/* Replaces mtgp32_init_by_str (mtgp32-fast.c:250-334). */
int mtgp32_gpu_init_by_str(mtgp32_gpu_t **out,
                           const mtgp32_params_fast_t *para, const char *str);
/* Replaces mtgp32_free (mtgp32-fast.c:342-344).  Synchronises the handle's
 * internal stream before freeing.  NULL is a no-op. */
void mtgp32_gpu_free(mtgp32_gpu_t *h);

/* n successive mtgp32_genrand_uint32 (mtgp32-fast.h:252-267) into dev_out. */
int mtgp32_gpu_fill_uint32(mtgp32_gpu_t *h, uint32_t *dev_out, size_t n,
                           void *stream);
/* n successive mtgp32_genrand_close1_open2 (mtgp32-fast.h:278-293). */
int mtgp32_gpu_fill_close1_open2(mtgp32_gpu_t *h, float *dev_out, size_t n,
                                 void *stream);
/* n successive mtgp32_genrand_close_open (mtgp32-fast.h:304-306). */
int mtgp32_gpu_fill_close_open(mtgp32_gpu_t *h, float *dev_out, size_t n,
                               void *stream);
/* n successive mtgp32_genrand_open_close (mtgp32-fast.h:317-319). */
int mtgp32_gpu_fill_open_close(mtgp32_gpu_t *h, float *dev_out, size_t n,
                               void *stream);
/* n successive mtgp32_genrand_open_open (mtgp32-fast.h:330-346). */
int mtgp32_gpu_fill_open_open(mtgp32_gpu_t *h, float *dev_out, size_t n,
                              void *stream);
/* Generic form of the five fills above; kind is an MTGP_KIND_* value.
 * Fills of 2^20 values or more (MEXP 11213 and 23209) are split into chunks
 * that start from GF(2)-jumped windows (made on the GPU first) and run on
 * many CTAs; such a fill may first wait for the split fill issued two calls
 * earlier on the same handle, the first one of a parameter set computes its
 * jump tables (tens of ms), and the first one with a new chunk length its
 * chunk polynomials (a synchronisation of `stream`).  Fills issued during
 * stream capture always run on one CTA. */
int mtgp32_gpu_fill(mtgp32_gpu_t *h, int kind, void *dev_out, size_t n,
                    void *stream);
/* Advance the state by n steps without writing output.  From 2^22 steps on
 * this is a GF(2) jump (X^n mod chi), not n generated steps; the state then
 * matches stepping except in the bits of word 0 that never reach an output. */
int mtgp32_gpu_skip(mtgp32_gpu_t *h, uint64_t n, void *stream);

/* Replaces mtgp32_fast_jump (mtgp32-fast-jump.c:51-79): jump_string is the
 * polynomial in the reference's hex form (digit k holds coefficients 4k..4k+3,
 * least significant bit first).  Runs on the GPU. */
int mtgp32_gpu_fast_jump(mtgp32_gpu_t *h, const char *jump_string,
                         void *stream);
/* Same jump with the polynomial in the reference's uint32-array form
 * (mtgp-calc-jump.hpp:67-91: bit j of word i is the coefficient of
 * X^(32i+j)), as stored in the jump tables (mtgp32-jump-table.h). */
int mtgp32_gpu_jump_array(mtgp32_gpu_t *h, const uint32_t *poly, int nwords,
                          void *stream);
/* Jump ahead by `steps` outputs (any 128-bit count, given as lo/hi words).
 * Uses the characteristic polynomial of the handle's parameter set
 * (computed once per set on the host by Berlekamp-Massey) and an
 * X^steps mod chi polynomial built on the host. */
int mtgp32_gpu_jump_steps(mtgp32_gpu_t *h, uint64_t steps_lo,
                          uint64_t steps_hi, void *stream);

/* Copy the device state into a reference struct whose status was allocated
 * by the reference (mtgp32_init) for the same parameter set; afterwards the
 * reference's genrand_* functions continue the sequence exactly.
 * Synchronous.  State mapping follows mtgp32-fast.h:165-183. */
int mtgp32_gpu_export(mtgp32_gpu_t *h, mtgp32_fast_t *dst);
/* Load the state (and parameters) of a reference struct into the handle. */
int mtgp32_gpu_import(mtgp32_gpu_t *h, const mtgp32_fast_t *src);
/* Live state window, oldest word first (size words), to / from host memory. */
int mtgp32_gpu_get_window_host(mtgp32_gpu_t *h, uint32_t *win, int size);
int mtgp32_gpu_set_window_host(mtgp32_gpu_t *h, const uint32_t *win, int size);

/* 64-bit twins: mtgp64-fast.c:99-142,156-339, mtgp64-fast.h:262-356,
 * mtgp64-fast-jump.c:51-79. */
int mtgp64_gpu_init(mtgp64_gpu_t **out, const mtgp64_params_fast_t *para,
                    uint64_t seed);
int mtgp64_gpu_init_by_array(mtgp64_gpu_t **out,
                             const mtgp64_params_fast_t *para,
                             const uint64_t *array, int length);
int mtgp64_gpu_init_by_str(mtgp64_gpu_t **out,
                           const mtgp64_params_fast_t *para, const char *str);
void mtgp64_gpu_free(mtgp64_gpu_t *h);
int mtgp64_gpu_fill_uint64(mtgp64_gpu_t *h, uint64_t *dev_out, size_t n,
                           void *stream);
int mtgp64_gpu_fill_close1_open2(mtgp64_gpu_t *h, double *dev_out, size_t n,
                                 void *stream);
int mtgp64_gpu_fill_close_open(mtgp64_gpu_t *h, double *dev_out, size_t n,
                               void *stream);
int mtgp64_gpu_fill_open_close(mtgp64_gpu_t *h, double *dev_out, size_t n,
                               void *stream);
int mtgp64_gpu_fill_open_open(mtgp64_gpu_t *h, double *dev_out, size_t n,
                              void *stream);
int mtgp64_gpu_fill(mtgp64_gpu_t *h, int kind, void *dev_out, size_t n,
                    void *stream);
int mtgp64_gpu_skip(mtgp64_gpu_t *h, uint64_t n, void *stream);
int mtgp64_gpu_fast_jump(mtgp64_gpu_t *h, const char *jump_string,
                         void *stream);
int mtgp64_gpu_jump_array(mtgp64_gpu_t *h, const uint32_t *poly, int nwords,
                          void *stream);
int mtgp64_gpu_jump_steps(mtgp64_gpu_t *h, uint64_t steps_lo,
                          uint64_t steps_hi, void *stream);
int mtgp64_gpu_export(mtgp64_gpu_t *h, mtgp64_fast_t *dst);
int mtgp64_gpu_import(mtgp64_gpu_t *h, const mtgp64_fast_t *src);
int mtgp64_gpu_get_window_host(mtgp64_gpu_t *h, uint64_t *win, int size);
int mtgp64_gpu_set_window_host(mtgp64_gpu_t *h, const uint64_t *win,
                               int size);

/* ========================================================================= */
/* Pools: many device-resident streams (bank, batched and serving paths)      */
/* ========================================================================= */
/* A pool holds `count` streams of one Mersenne exponent.  Stream i uses
 * parameter set params[param_idx ? param_idx[i] : i] and its window stays in
 * HBM between calls.  The reference has no counterpart object; its CUDA
 * samples keep the same data in mtgp32_kernel_status_t arrays
 * (cuda-sample/mtgp32-cuda.cu:43-45) and launch one CTA per generator. */
typedef struct mtgp32_gpu_pool mtgp32_gpu_pool_t;
typedef struct mtgp64_gpu_pool mtgp64_gpu_pool_t;

/* One unit of batched work: advance stream `stream` by `skip` values
 * without output, then produce `count` values of `kind` (MTGP_KIND_*, or
 * -1 = advance without output) at byte offset `out_offset` of the output
 * buffer (a multiple of the value size).  Items naming the same stream are
 * applied in array order.  For MEXP 11213 and 23209, a skip (or an
 * advance-only item) of 2^17 values or more is done by a GF(2) jump (X^skip
 * mod chi, inside the batched kernel) instead of generation; for the other
 * exponents skips are generated, and a skip above 2^34 is rejected with
 * MTGP_ERR_UNSUPPORTED. */
typedef struct mtgp_work_item {
    uint32_t stream;
    int32_t kind;
    uint64_t count;
    uint64_t out_offset;
    uint64_t skip;
} mtgp_work_item_t;

/* A prepared batch: descriptors uploaded once, launched many times. */
typedef struct mtgp_gpu_plan mtgp_gpu_plan_t;

/* Seeded pool: stream i = mtgp32_init(params[pidx[i]], seeds[i]). */
int mtgp32_gpu_pool_create(mtgp32_gpu_pool_t **out,
                           const mtgp32_params_fast_t *params, int nparams,
                           const int *param_idx, const uint32_t *seeds,
                           int count);
/* Pools seeded by key schedules, on the device (one thread per stream):
 * stream i = mtgp32_init_by_array(params[pidx[i]], keys + key_offsets[i],
 * key_offsets[i+1] - key_offsets[i]) (mtgp32-fast.c:151-235), or
 * mtgp32_init_by_str(params[pidx[i]], strs[i]) (mtgp32-fast.c:250-334, the
 * bytes read as signed char).  key_offsets has count + 1 entries. */
int mtgp32_gpu_pool_create_by_array(mtgp32_gpu_pool_t **out,
                                    const mtgp32_params_fast_t *params,
                                    int nparams, const int *param_idx,
                                    const uint32_t *keys,
                                    const uint64_t *key_offsets, int count);
int mtgp32_gpu_pool_create_by_str(mtgp32_gpu_pool_t **out,
                                  const mtgp32_params_fast_t *params,
                                  int nparams, const int *param_idx,
                                  const char *const *strs, int count);
/* Substream pool: stream j = (para, seed) jumped ahead by j * step, where
 * jump_table row k (nwords words each) is X^(4^k * step) mod chi, the layout
 * of the reference's jump tables (cuda-sample/mtgp32-jump-table.h:6-13).
 * count <= 4^rows.  The jumps run on the GPU: the same rows in the same
 * order as the reference's table walk (cuda-sample/mtgp32-jump-kernel.cuh:
 * 383-423), so the windows are identical to it, but made by doubling (level
 * k jumps windows [0, 2^k) into [2^k, 2^(k+1))), one jump per substream. */
int mtgp32_gpu_pool_create_substreams(mtgp32_gpu_pool_t **out,
                                      const mtgp32_params_fast_t *para,
                                      uint32_t seed, int count,
                                      const uint32_t *jump_table, int rows,
                                      int nwords, void *stream);
void mtgp32_gpu_pool_free(mtgp32_gpu_pool_t *p);
int mtgp32_gpu_pool_size(const mtgp32_gpu_pool_t *p);
/* Plain path, one launch for the whole pool (one CTA per stream): every
 * stream produces n_per_stream values at dev_out + i * n_per_stream. */
int mtgp32_gpu_pool_fill(mtgp32_gpu_pool_t *p, int kind, void *dev_out,
                         size_t n_per_stream, void *stream);
/* Plain path for one stream (one launch, one CTA). */
int mtgp32_gpu_pool_fill_stream(mtgp32_gpu_pool_t *p, int s, int kind,
                                void *dev_out, size_t n, void *stream);
/* Batched path: all items in one persistent launch. */
int mtgp32_gpu_pool_submit(mtgp32_gpu_pool_t *p, const mtgp_work_item_t *items,
                           int nitems, void *dev_out, void *stream);
int mtgp32_gpu_pool_plan(mtgp32_gpu_pool_t *p, const mtgp_work_item_t *items,
                         int nitems, mtgp_gpu_plan_t **plan);
/* Refill an existing plan of this pool with new items, keeping (and only
 * growing) its device buffers.  The plan must not be in use on the GPU. */
int mtgp32_gpu_pool_replan(mtgp32_gpu_pool_t *p, const mtgp_work_item_t *items,
                           int nitems, mtgp_gpu_plan_t *plan);
/* Jump stream s by a polynomial (uint32-array form). */
int mtgp32_gpu_pool_jump_array(mtgp32_gpu_pool_t *p, int s,
                               const uint32_t *poly, int nwords, void *stream);
/* X^steps[j] mod chi of parameter set `param_set`, for j < n, computed on the
 * GPU in the uint32-array form of jump_array: mexp/32 + 1 words each at
 * dev_out + j * (mexp/32 + 1).  steps is host memory.  Products of at most
 * eight byte-window table polynomials (the table is made on the GPU at the
 * first call for the parameter set, synchronously); a few exponents spread
 * over many CTAs, many run one per CTA.  Replaces NTL's PowerXMod
 * (mtgp-calc-jump.hpp:135-162); batched work items with uncached long skips
 * use the same products.  MTGP_ERR_UNSUPPORTED if the polynomials are too
 * long for the product kernel's shared memory. */
int mtgp32_gpu_pool_jump_polys(mtgp32_gpu_pool_t *p, int param_set,
                               const uint64_t *steps, int n, uint32_t *dev_out,
                               void *stream);
/* All windows, count * size words, stream-major (synchronous). */
int mtgp32_gpu_pool_get_windows_host(mtgp32_gpu_pool_t *p, uint32_t *win,
                                     size_t nwords);
int mtgp32_gpu_pool_set_windows_host(mtgp32_gpu_pool_t *p,
                                     const uint32_t *win, size_t nwords);
int mtgp32_gpu_pool_export(mtgp32_gpu_pool_t *p, int s, mtgp32_fast_t *dst);

int mtgp64_gpu_pool_create(mtgp64_gpu_pool_t **out,
                           const mtgp64_params_fast_t *params, int nparams,
                           const int *param_idx, const uint64_t *seeds,
                           int count);
int mtgp64_gpu_pool_create_by_array(mtgp64_gpu_pool_t **out,
                                    const mtgp64_params_fast_t *params,
                                    int nparams, const int *param_idx,
                                    const uint64_t *keys,
                                    const uint64_t *key_offsets, int count);
int mtgp64_gpu_pool_create_by_str(mtgp64_gpu_pool_t **out,
                                  const mtgp64_params_fast_t *params,
                                  int nparams, const int *param_idx,
                                  const char *const *strs, int count);
int mtgp64_gpu_pool_create_substreams(mtgp64_gpu_pool_t **out,
                                      const mtgp64_params_fast_t *para,
                                      uint64_t seed, int count,
                                      const uint32_t *jump_table, int rows,
                                      int nwords, void *stream);
void mtgp64_gpu_pool_free(mtgp64_gpu_pool_t *p);
int mtgp64_gpu_pool_size(const mtgp64_gpu_pool_t *p);
int mtgp64_gpu_pool_fill(mtgp64_gpu_pool_t *p, int kind, void *dev_out,
                         size_t n_per_stream, void *stream);
int mtgp64_gpu_pool_fill_stream(mtgp64_gpu_pool_t *p, int s, int kind,
                                void *dev_out, size_t n, void *stream);
int mtgp64_gpu_pool_submit(mtgp64_gpu_pool_t *p, const mtgp_work_item_t *items,
                           int nitems, void *dev_out, void *stream);
int mtgp64_gpu_pool_plan(mtgp64_gpu_pool_t *p, const mtgp_work_item_t *items,
                         int nitems, mtgp_gpu_plan_t **plan);
int mtgp64_gpu_pool_replan(mtgp64_gpu_pool_t *p, const mtgp_work_item_t *items,
                           int nitems, mtgp_gpu_plan_t *plan);
int mtgp64_gpu_pool_jump_array(mtgp64_gpu_pool_t *p, int s,
                               const uint32_t *poly, int nwords, void *stream);
int mtgp64_gpu_pool_jump_polys(mtgp64_gpu_pool_t *p, int param_set,
                               const uint64_t *steps, int n, uint32_t *dev_out,
                               void *stream);
int mtgp64_gpu_pool_get_windows_host(mtgp64_gpu_pool_t *p, uint64_t *win,
                                     size_t nwords);
int mtgp64_gpu_pool_set_windows_host(mtgp64_gpu_pool_t *p,
                                     const uint64_t *win, size_t nwords);
int mtgp64_gpu_pool_export(mtgp64_gpu_pool_t *p, int s, mtgp64_fast_t *dst);

/* Autotuner (no reference counterpart): builds a plan for each candidate
 * configuration -- generation core (four words per thread in 64-thread CTAs
 * with 128-bit stores, or one word per thread in 256-thread CTAs), the chunk
 * length used to split long requests, and the grid size -- times each on
 * these items and this output buffer (median of `reps` launches on `stream`),
 * and returns the fastest.  The pool's windows are restored before every
 * trial and at the end, so the pool is left unchanged.  `report` (optional)
 * receives one line per candidate. */
int mtgp32_gpu_pool_autotune(mtgp32_gpu_pool_t *p, const mtgp_work_item_t *items,
                             int nitems, void *dev_out, void *stream, int reps,
                             mtgp_gpu_plan_t **plan, char *report, int report_cap);
int mtgp64_gpu_pool_autotune(mtgp64_gpu_pool_t *p, const mtgp_work_item_t *items,
                             int nitems, void *dev_out, void *stream, int reps,
                             mtgp_gpu_plan_t **plan, char *report, int report_cap);

/* Launch a prepared batch (one persistent kernel).  Capturable. */
int mtgp_gpu_plan_launch(mtgp_gpu_plan_t *plan, void *dev_out, void *stream);
/* Same launch through a CUDA graph, captured on first use for this
 * dev_out and replayed afterwards. */
int mtgp_gpu_plan_graph_launch(mtgp_gpu_plan_t *plan, void *dev_out,
                               void *stream);
/* Bytes of output the plan writes (max over items of offset + size). */
uint64_t mtgp_gpu_plan_output_bytes(const mtgp_gpu_plan_t *plan);
/* Tasks of the launch after splitting, and the chunk length used to split
 * long requests (0 = none split). */
int mtgp_gpu_plan_info(const mtgp_gpu_plan_t *plan, int64_t *tasks,
                       int64_t *chunk);
/* The plan's configuration, the first n of: [0] tasks, [1] split chunk
 * length (0 = none), [2] generation core (1, 2 or 4), [3] grid (0 = all
 * resident CTAs), [4] kernels one launch runs, [5] 1 if tasks start with
 * in-kernel jumps, [6] tasks that start from a window jumped ahead of the
 * launch (by jump parts, before the persistent kernel), [7] 1 if those
 * tasks run in a second launch beside the first ("jump_overlap").  Passing
 * [1]-[3] and [7] to mtgp32/64_gpu_pool_set_tuning ("core", "split_chunk"
 * (-1 for 0), "batch_grid", "jump_overlap") makes plans of the same kind. */
int mtgp_gpu_plan_describe(const mtgp_gpu_plan_t *plan, int64_t *values,
                           int n);
/* Tuning knobs (no reference counterpart; the autotuner and tests use
 * them).  Every pool and single generator carries its own knobs:
 * mtgp_gpu_set_tuning sets the process-wide defaults that pools and
 * generators created afterwards start from (existing handles keep theirs),
 * and the *_set_tuning calls below change one handle's knobs for the plans
 * and fills it makes afterwards.  Tuning one handle never changes another's
 * plans, so a server's scheduler thread is not affected by tuning calls on
 * other threads.  A handle's own knobs follow the handle's single-owner
 * rule: do not change them while another thread plans with the handle.
 * Keys:
 *   "split_chunk"  0 = automatic, < 0 = never split, > 0 = chunk length
 *   "batch_grid"   0 = one CTA per resident slot, > 0 = that many CTAs
 *   "core"         32-bit generation core: 2 = two adjacent words per
 *                  thread (default), 4 = four, 1 = one word per thread; plans
 *                  whose items mix output kinds use the one-word core
 *   "poly_window"  bits per table window of the GPU's polynomial products
 *                  (jump polynomials): 0 = automatic (4 where the table
 *                  fits in shared memory, else 2), 2 or 4
 *   "single_chunk" chunk length of a split single-generator fill (fills of
 *                  at least 2^20 values): 0 = automatic, > 0 = that length
 *   "jump_parts"   jumps made ahead of a batched launch (the chunk starts of
 *                  such a fill, and batched tasks that start with one jump):
 *                  CTAs per jump, 0 = automatic (4), > 0 = that many (at
 *                  most one per tap chunk of the jump kernel); -1 = such
 *                  jumps run inside the batched kernel instead
 *   "jump_overlap" 0 = the jump parts run before the persistent launch;
 *                  1 = they run on a side stream of the plan, followed there
 *                  by a second persistent launch of the tasks that start
 *                  from their windows, while the caller's stream runs the
 *                  other tasks (fork and join by events) */
int mtgp_gpu_set_tuning(const char *key, int64_t value);
int mtgp32_gpu_pool_set_tuning(mtgp32_gpu_pool_t *pool, const char *key,
                               int64_t value);
int mtgp64_gpu_pool_set_tuning(mtgp64_gpu_pool_t *pool, const char *key,
                               int64_t value);
int mtgp32_gpu_gen_set_tuning(mtgp32_gpu_t *gen, const char *key,
                              int64_t value);
int mtgp64_gpu_gen_set_tuning(mtgp64_gpu_t *gen, const char *key,
                              int64_t value);
void mtgp_gpu_plan_free(mtgp_gpu_plan_t *plan);

/* ========================================================================= */
/* Batched generation without any allocation                                  */
/* ========================================================================= */
/* For callers that cannot allocate device memory: engines whose device memory
 * is all reserved up front in their own arena or under a hard budget, and
 * plug-ins that may only use the buffers a host application hands them.  No
 * counterpart in the reference.
 *
 * The caller passes the stream windows and the output.  dev_windows holds
 * nstreams windows (MEXP 11213/23209/44497), each mexp/32+1 words oldest word
 * first, at a stride of roundup(mexp/32+1, 32) words; they are advanced in
 * place.  Stream s uses params[param_idx ? param_idx[s] : s] (or params[0]
 * when nparams != nstreams).  Items follow mtgp32_gpu_pool_submit's rules,
 * without long-request splitting.  The kernel's descriptors go into one
 * fixed array in device memory inside the library (about 116 KB, held by
 * every GPU that loads the library until the process exits): at most 16
 * parameter sets and 2048 items per call, larger requests are rejected with
 * MTGP_ERR_INVALID.  The first call on a device looks up the array's device
 * address and keeps it for the life of the process, so it should come
 * before any stream capture, and no call may follow a cudaDeviceReset of
 * that device.  Every call overwrites the array: calls whose GPU work
 * overlaps (other streams, other host threads) race and must be serialised
 * by the caller.  Each call first waits for all work already queued on
 * `stream` (a host-side synchronisation: the descriptors come from host
 * memory, and the previous call may still be reading the array), uploads
 * the descriptors and returns; generation then runs on `stream`.  On a
 * stream that is being captured, which cannot be synchronised, it returns
 * MTGP_ERR_UNSUPPORTED and leaves the stream untouched. */
int mtgp32_gpu_batch_noalloc(const mtgp32_params_fast_t *params, int nparams,
                             const int *param_idx, uint32_t *dev_windows,
                             int nstreams, const mtgp_work_item_t *items,
                             int nitems, void *dev_out, void *stream);

/* ========================================================================= */
/* Serving loop: continuous batching over resident pools                      */
/* ========================================================================= */
/* No counterpart in the reference (its generators are filled by the caller,
 * one launch per request).  A server owns a device output arena of
 * `budget_bytes` (the memory budget) and a scheduler thread that admits
 * pending requests first-come-first-served into batches of at most
 * `max_batch` requests (and an eighth of the budget, up to half under a
 * backlog), keeps up to `slots` (at most
 * 256) batches in flight on their own CUDA streams, and copies each result
 * to its destination when the batch completes.  A batch's outputs take one
 * block of the arena, placed in admission order; results kept in the arena
 * (mtgp_server_submit without destination) hold their part of a block until
 * released, so long-kept results fragment the arena.  Requests of one
 * stream run in submission order (a batch that holds a stream runs on the
 * GPU after the stream's earlier batches); a request's values depend only
 * on its stream's position, so they are the same alone and in any mix.
 * While a server runs, its pools must not be used otherwise. */
typedef struct mtgp_server mtgp_server_t;

/* One request of a trace (mtgp_server_replay). */
typedef struct mtgp_request {
    int32_t pool;     /* 0 = the 32-bit pool, 1 = the 64-bit pool          */
    uint32_t stream;  /* stream of that pool                               */
    int32_t kind;     /* MTGP_KIND_*, or -1 = advance only                 */
    int32_t pad_;
    uint64_t skip;    /* values skipped first (GF(2) jump when large)      */
    uint64_t count;   /* values produced                                   */
    void *dst;        /* device or host destination, or NULL = discard     */
} mtgp_request_t;
/* (In a replayed trace a request without destination is discarded when it
 * completes; mtgp_server_submit keeps such results instead.) */

/* Either pool may be NULL (not both).  The pools must outlive the server. */
int mtgp_server_create(mtgp_server_t **out, mtgp32_gpu_pool_t *p32,
                       mtgp64_gpu_pool_t *p64, uint64_t budget_bytes,
                       int slots, int max_batch);
/* Queue a request (thread-safe).  Tickets count from 1.  A request whose
 * output alone exceeds the budget is rejected with MTGP_ERR_BUDGET.  With
 * dst == NULL the result stays in the server's device arena (zero copy):
 * mtgp_server_result gives its address once the request is done, and
 * mtgp_server_release returns the space to the budget. */
int mtgp_server_submit(mtgp_server_t *s, int pool, uint32_t stream, int kind,
                       uint64_t skip, uint64_t count, void *dst,
                       uint64_t *ticket);
/* Device address and size of a finished request's result kept in the arena
 * (valid until mtgp_server_release or mtgp_server_destroy). */
int mtgp_server_result(mtgp_server_t *s, uint64_t ticket, void **dev_ptr,
                       uint64_t *bytes);
int mtgp_server_release(mtgp_server_t *s, uint64_t ticket);
/* Remove a request that has not been admitted yet; its status becomes
 * MTGP_ERR_BUSY.  Fails with MTGP_ERR_INVALID once it is admitted.  (A
 * request is not admitted while the arena, less the results kept in it and
 * the batches admitted but not yet placed, cannot hold it.) */
int mtgp_server_cancel(mtgp_server_t *s, uint64_t ticket);
/* Wait until a request is done (its destination holds the result);
 * `status` receives MTGP_OK or the error it ended with (a request whose batch
 * failed may still have advanced its stream). */
int mtgp_server_wait(mtgp_server_t *s, uint64_t ticket, double timeout_s,
                     int *status);
/* Wait until every submitted request is done. */
int mtgp_server_drain(mtgp_server_t *s, double timeout_s);
/* Per-ticket latency in seconds (submission to completion; -1 while
 * pending) and status, for tickets 1..min(cap, submitted); n = submitted. */
int mtgp_server_results(mtgp_server_t *s, double *latency, int *status,
                        uint64_t cap, uint64_t *n);
int mtgp_server_stats(mtgp_server_t *s, uint64_t *completed, uint64_t *bytes,
                      uint64_t *batches);
/* Host time spent so far, in seconds: [0] admitting requests (the
 * scheduler thread), [1] planning and launching batches (with the waits for
 * arena space and for the launches of earlier batches of the same streams)
 * and [2] retiring them (summed over the slots' worker threads, which run
 * in parallel), [3] the scheduler waiting for work, [4] the planning part of
 * [1] (the first n of these five). */
int mtgp_server_profile(mtgp_server_t *s, double *seconds, int n);
/* Submit n requests at their arrival times (seconds after the call starts),
 * then drain; wall_s receives the elapsed time. */
int mtgp_server_replay(mtgp_server_t *s, const mtgp_request_t *reqs,
                       const double *arrival_s, int n, double *wall_s);
/* Drains, stops the scheduler and frees the arena (the pools stay). */
void mtgp_server_destroy(mtgp_server_t *s);

#if defined(__cplusplus)
}
#endif
#endif /* MTGP_GPU_H */
