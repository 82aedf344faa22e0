/*
 * gbx_dltc.h -- C ABI of the DLTC executor: the Multiplication / Summation
 * tile loops of DLTC's task functions and its residual tables (CCD-T2,
 * CCSD-T1, CCSD-T2) on the GPU.
 *
 * A DLTC tensor is held as Global Arrays hold it (DLTC/dltc_tensor.cc:14-40):
 * dense, row-major over the tensor's index order, every hole index of extent
 * O and every particle index of extent V, cut into tiles of wbO / wbV
 * elements per index.  Index names are the IndexName values of
 * DLTC/param.h: names below nocc_names are holes (h1..h12 = 0..11 with
 * nocc_names = 12; H1..H6 = 0..5 with 6 in the reference's check build),
 * the rest particles.  Conventions as in gbx.h: int status, messages via
 * gbx_last_error(), streams as void*.
 */
#ifndef GBX_DLTC_H
#define GBX_DLTC_H
#include <stdint.h>

#include "gbx.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GBX_DLTC_MAX_NAMES 24 /* IndexName values 0 .. 23 */
#define GBX_DLTC_MUL 0
#define GBX_DLTC_SUM 1

typedef struct {
    int O, V;         /* extents of hole / particle indices */
    int wbO, wbV;     /* tile widths (O % wbO == 0, V % wbV == 0) */
    int nocc_names;   /* index names below this are holes */
} gbx_dltc_dims;

/* The index orders of a Multiplication tC += coef * tA * tB as its
 * constructor derives them (DLTC/expr.cc:13-67): m = names of A only,
 * n = names of B only, k = names of both, each sorted by name; the tiles are
 * transposed to at = m + k, bt = k + n, and the product ct = m + n.  Host
 * only.  Any output pointer may be NULL. */
GBX_API int gbx_dltc_mul_orders(int rA, const int* idA, int rB, const int* idB, int* m_ids, int* nm, int* n_ids,
                                int* nn, int* k_ids, int* nk);

/* task_mul over the tile ranges lo[name] <= tile < hi[name] (host arrays of
 * GBX_DLTC_MAX_NAMES; both NULL = every tile): for every C tile of the range,
 * C += coef * sum over the contracted tiles of A * B, with A and B transposed
 * into at / bt order and the product back from ct order.  d_A, d_B, d_C are
 * whole tensors on the device.  mode GBX_MODE_FP64 (FP64 GEMM) or
 * GBX_MODE_SPLIT (split-precision engine, default slices).  Stream-ordered
 * temporaries; with the split engine the call waits for the stream.
 * Replaces: void task_mul(int id, int lmap[], int hmap[])  DLTC/task.cc:83-137
 * (and with full ranges exec(MUL, id) of one expression, DLTC/exec.cc:42-111). */
GBX_API int gbx_dltc_task_mul(double coef, int rC, const int* idC, double* d_C, int rA, const int* idA,
                              const double* d_A, int rB, const int* idB, const double* d_B, const gbx_dltc_dims* dims,
                              const int* lo, const int* hi, int mode, void* stream);

/* task_sum over the tile ranges: C += coef * A transposed to C's order.
 * Replaces: void task_sum(int id, int lmap[], int hmap[])  DLTC/task.cc:51-81. */
GBX_API int gbx_dltc_task_sum(double coef, int rC, const int* idC, double* d_C, int rA, const int* idA,
                              const double* d_A, const gbx_dltc_dims* dims, const int* lo, const int* hi,
                              void* stream);

/* ---- residual tables ----------------------------------------------------- */

#define GBX_DLTC_CCD_T2 0  /* DLTC/ccd-t2.cc:3-134   (ccd_t2)  */
#define GBX_DLTC_CCSD_T1 1 /* DLTC/ccsd-t1.cc:3-165  (ccsd_t1) */
#define GBX_DLTC_CCSD_T2 2 /* DLTC/ccsd-t2.cc:3-310  (ccsd_t2) */

/* One expression of a table, in execution order (layer by layer, and within
 * a layer in the order of the reference's exec calls). */
typedef struct {
    int kind;          /* GBX_DLTC_MUL (m[index]) or GBX_DLTC_SUM (s[index]) */
    int index;
    int layer;         /* 0-based dependency layer (a Barrier between layers) */
    int c, a, b;       /* tensor numbers (enum TensorName order); b = -1 for a Summation */
    int rc, ra, rb;
    int idc[4], ida[4], idb[4];
    double coef;
} gbx_dltc_expr;

/* The table's expressions (*nexpr in: capacity, out: count; exprs may be
 * NULL to query) and tensors: per tensor 5 ints in types (rank, then 0 = hole
 * / 1 = particle per index, -1 padding) and its name in names (name_len chars
 * each); *ntensors in: capacity, out: count.  Host only. */
GBX_API int gbx_dltc_table(int which, gbx_dltc_expr* exprs, int* nexpr, int* types, int* ntensors, char* names,
                           int name_len);

typedef struct gbx_dltc_program gbx_dltc_program;

/* A table bound to device tensors of the given dims, zeroed (as GA_Zero
 * leaves them), with every expression prepared once: transposes, GEMM (mode
 * GBX_MODE_FP64 or GBX_MODE_SPLIT) and one shared workspace.
 * Replaces the setup half of ccd_t2 / ccsd_t1 / ccsd_t2 (Tensor2/Tensor4 +
 * allocGA + the Multiplication / Summation constructors). */
GBX_API int gbx_dltc_program_create(int which, const gbx_dltc_dims* dims, int mode, gbx_dltc_program** out);
/* Device buffer of tensor t (dense, index order of its table entry). */
GBX_API int gbx_dltc_program_tensor(gbx_dltc_program* p, int tensor, double** d_data, int64_t* elems);
/* Enqueue expressions [first, first + count) of the execution order
 * (count < 0: to the end) on stream.  All of them = the layers of the
 * table one after the other (the Barriers become stream order).
 * Replaces the exec / gtc_process half of ccd_t2 / ccsd_t1 / ccsd_t2. */
GBX_API int gbx_dltc_program_run(gbx_dltc_program* p, int first, int count, void* stream);
/* GBX_ETIMEOUT if a bounded device wait of the split engine ran out (syncs). */
GBX_API int gbx_dltc_program_check(gbx_dltc_program* p);
/* 2 * M * N * K summed over the Multiplications. */
GBX_API double gbx_dltc_program_flops(const gbx_dltc_program* p);
GBX_API int gbx_dltc_program_destroy(gbx_dltc_program* p);

#ifdef __cplusplus
}
#endif
#endif /* GBX_DLTC_H */
