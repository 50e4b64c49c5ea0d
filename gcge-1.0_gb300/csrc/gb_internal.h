/*
 * gb_internal.h -- internal interface between the C host driver (gb_solver.c,
 * gb_ops_table.c) and the CUDA sources (gb_blas.cu, gb_dense.cu, gb_api.cu).
 *
 * Storage conventions
 *  - Multivector: row-major n x ncols block in HBM, element (row r, column c)
 *    at d[r*ld + c]; ld = ncols rounded up to an even count so that column
 *    offsets that are even stay 16-byte aligned. A column range is addressed by
 *    offsetting the base pointer (d + c0) and keeping ld.
 *  - Small dense matrices (projected matrix, coefficients, Gram blocks) are
 *    column-major, as in the reference, and stay in device memory.
 */
#ifndef GB_INTERNAL_H
#define GB_INTERNAL_H

#include <cuda_runtime.h>
#include "gcge_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GB_PROF_SLOTS 4096
/* kernel classes of the profiling mode (order of GCGE_GPU_ProfileRead) */
enum { GB_K_SPMM64, GB_K_SPMM32, GB_K_GRAM, GB_K_LINCOMB, GB_K_BCGVEC, GB_K_BLAS1, GB_K_DENSE, GB_K_EIG,
       GB_K_REDUCE, GB_K_SPMMPAIR, GB_PROF_CLASSES };

/* a device block held by the context's cache (gb_dev_alloc / gb_dev_free) */
typedef struct {
    void *p;
    size_t bytes;
    int used;
} gb_block;

struct gcge_gpu_ctx {
    int device;
    int num_sms;
    cudaStream_t stream;
    /* reduction and small-matrix scratch (grown on demand, outside timed loops) */
    double *scratch;
    size_t scratch_cap;        /* doubles */
    double *coef;              /* device staging of host coefficient arrays */
    size_t coef_cap;           /* doubles */
    double *pinned;            /* pinned host staging */
    size_t pinned_cap;         /* doubles */
    int err;                   /* sticky first error */
    long long launches;        /* kernel launches issued through this context */
    long long spmm_launches;
    /* profiling (GCGE_GPU_ProfileEnable): events around each launch, per class */
    int prof;
    int prof_used;
    cudaEvent_t *prof_ev;      /* 2 * GB_PROF_SLOTS */
    int *prof_cls;
    double *prof_bytes, *prof_flops;
    double cls_ms[GB_PROF_CLASSES], cls_bytes[GB_PROF_CLASSES], cls_flops[GB_PROF_CLASSES];
    long long cls_launches[GB_PROF_CLASSES];
    /* dense FP64 contractions (Gram, linear combination) on the bf16 tensor cores
     * with an error-free digit splitting (1, default) or on the FP64 pipe (0) */
    int tc;
    int *iscratch;
    size_t iscratch_cap;
    void *ozbuf;               /* pre-split digit planes of small operands */
    size_t ozbuf_cap;          /* bytes */
    int *dev_err;              /* device word: set by a kernel whose bounded wait ran out */
    int tc_stall;              /* test hook: the next tensor-core launch withholds an arrival */
    /* FP64 SpMM in FP32-pair arithmetic (1; set by the mixed solver form) or on the
     * FP64 pipe (0, default) */
    int spmm_pair;
    float *pairbuf;            /* X split into (hi, lo) FP32 pairs */
    size_t pairbuf_cap;        /* floats */
    int *dev_pairflag;         /* device word: epoch of the last split that met |x| >= 2^100 */
    int pair_epoch;
    gb_block *blk;             /* workspace blocks kept for later solves on this context */
    int nblk, blk_cap;
};

struct gcge_gpu_mat {
    gcge_gpu_ctx *ctx;
    int n, nnz;
    int *rp, *ci;              /* device CSR structure */
    double *v;                 /* device FP64 values */
    float *v32;                /* device FP32 values (mixed precision) or NULL */
    double max_row_nnz;
    double *dinv;              /* 1 / diag(A) for the Jacobi preconditioner (lazy) or NULL */
    float *dinv32;             /* the same in FP32 */
    float *vpair;              /* values x 2^-s as (hi, lo) FP32 pairs (lazy) or NULL */
    int *pair_meta;            /* device: [0..1] max |value| bits, [2] the exponent s */
    int *lrows;                /* device: rows with more than GB_LONG_ROW entries (FP32 matrices) */
    int nlong;                 /* their count */
    long nnz_long;             /* their entries */
};

/* rows longer than this are shared by a whole block in the FP32 block-CG SpMM */
#define GB_LONG_ROW 64

struct gcge_gpu_mv {
    gcge_gpu_ctx *ctx;
    int n, ncols;
    long ld;
    double *d;
};

/* device workspace through the context's block cache: a released block is kept
 * and handed to a later request of between its size and half of it (best fit);
 * all are freed by GCGE_GPU_Finalize (and unused ones when cudaMalloc fails) */
int  gb_dev_alloc(gcge_gpu_ctx *ctx, void **p, size_t bytes);
void gb_dev_free(gcge_gpu_ctx *ctx, void *p);

/* profiling hooks around a launch: class, algorithmic bytes and flops */
void gb_prof_begin(gcge_gpu_ctx *ctx, int cls, double bytes, double flops);
void gb_prof_end(gcge_gpu_ctx *ctx);

/* record the first error on the context; returns st */
int gb_fail(gcge_gpu_ctx *ctx, int st);
int gb_check_launch(gcge_gpu_ctx *ctx);
/* ensure ctx->scratch holds at least n doubles */
int gb_scratch(gcge_gpu_ctx *ctx, size_t n);
int gb_coef(gcge_gpu_ctx *ctx, size_t n);
int gb_pinned(gcge_gpu_ctx *ctx, size_t n);
int gb_iscratch(gcge_gpu_ctx *ctx, size_t n);
int gb_ozbuf(gcge_gpu_ctx *ctx, size_t bytes);
int gb_check_device_error(gcge_gpu_ctx *ctx);
/* FP64-accurate Gram on the tensor cores (gb_ozaki.cu); exps: int[k1 + k2] */
int gb_gram_tc(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *V, long ldv, const double *W, long ldw,
               double *a_dev, int lda, int sym, int *exps);
/* FP64-accurate Y = alpha X C + beta Y on the tensor cores (gb_ozaki.cu), for k1 where
 * gb_lincomb_tc_ok(k1) holds */
int gb_lincomb_tc_ok(int k1);
int gb_lincomb_tc_inplace_ok(int k1, int k2);
/* 1 when gb_lincomb may write Y over columns of X (same rows, same ld) */
int gb_lincomb_inplace_ok(const gcge_gpu_ctx *ctx, int k1, int k2);
int gb_lincomb_tc(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *X, long ldx, const double *C, int ldc,
                  double alpha, double beta, double *Y, long ldy, int upper);

/* ------------------------------------------------------------ gb_blas.cu */
/* Y[:, 0:k] = alpha_c * (A X[:, 0:k]) + beta * Y, alpha_c = alpha * (alpha_col ? alpha_col[c] : 1).
 * ncols_dev (optional): device int; columns >= *ncols_dev are left untouched. */
int gb_spmm(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const double *X, long ldx, double *Y, long ldy,
            int k, double alpha, const double *alpha_col, double beta, const int *ncols_dev);
/* A X and B X (B may be NULL) from one split of X in the FP32-pair form */
int gb_spmm_ab(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, const double *X, long ldx,
               double *YA, double *YB, long ldy, int k);
int gb_spmm32(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const float *X, long ldx, float *Y, long ldy,
              int k, const int *ncols_dev);
/* y = a x + b y on an n x k block, CSR_VecAxpby special cases */
int gb_axpby(gcge_gpu_ctx *ctx, int n, int k, double a, const double *X, long ldx, double b,
             double *Y, long ldy);
/* Y[:, c] = X[:, idx[c]] * scale(c); scale from eval[idx[c]]: mode 0 -> 1,
 * mode 1 -> (|l| <= 1 ? 1 : 1/l) (initial guess of ComputeW) */
int gb_gather_cols(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const int *idx_dev,
                   double *Y, long ldy, const double *eval_dev, int mode);
/* per-column dots out[c] = sum_r X[r,c] Y[r,c] (deterministic two-stage) */
int gb_col_dots(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const double *Y, long ldy,
                double *out_dev);
/* residual norms for the convergence test: for c < k with l = eval[idx[c]]
 * out[3c+0] = ||AX_c - l BX_c||^2, out[3c+1] = ||X_c||^2, out[3c+2] = ||BX_c||^2
 * (BX == NULL means B = I); bnorm != 0 forms only the first and the last (the
 * middle slot then repeats the last), otherwise only the first two (the last
 * repeats the middle) */
int gb_residual_norms(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const double *AX,
                      long ldax, const double *BX, long ldbx, const double *eval_dev, const int *idx_dev,
                      double *out_dev, int bnorm);
/* a[i + j*lda] = sum_r V[r,i] W[r,j], i < k1, j < k2 (sym: i <= j computed, mirrored) */
int gb_gram(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *V, long ldv, const double *W, long ldw,
            double *a_dev, int lda, int sym);
/* Y[:, j] = alpha * sum_i X[:, i] C[i + j*ldc] + beta * Y[:, j]; upper != 0 asserts C[i, j] = 0 for i > j */
int gb_lincomb(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *X, long ldx, const double *C_dev,
               int ldc, double alpha, double beta, double *Y, long ldy, int upper);
int gb_fill_random(gcge_gpu_ctx *ctx, int n, int k, double *X, long ldx, int col0,
                   unsigned long long seed);
int gb_convert_d2f(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, float *Y, long ldy);
int gb_convert_f2d(gcge_gpu_ctx *ctx, int n, int k, const float *X, long ldx, double *Y, long ldy);
/* zero rows flagged by the Dirichlet rule of CSR_SetDirichletBoundary */
int gb_dirichlet_zero(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, int k,
                      double *X, long ldx);
/* strided single-vector helpers (GCGE_OPS single-vector members) */
int gb_frobenius(gcge_gpu_ctx *ctx, int m, int n, const double *a, int lda, double *out_dev);

/* block CG on FP64 or FP32 data, all control state on the device */
typedef struct {
    int n, k, max_it, precision;
    double rate;
    int rhs_is_residual;       /* RHS already holds RHS - A X: skip the initial product */
    const double *dinv;        /* Jacobi preconditioner 1/diag(A) (FP64 rounds) or NULL: plain CG */
    const float *dinv32;       /* the same for the FP32 rounds */
    int residual_unused;       /* the caller does not read RHS afterwards: the mixed
                                  form skips writing the final residual back into it */
} gb_bcg_args;
/* 1 / diag(A) in FP64 and FP32, computed once per matrix values (a zero or missing
 * diagonal entry gives 1) */
int gb_mat_dinv(gcge_gpu_ctx *ctx, gcge_gpu_mat *A);
int gb_bcg(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, double *RHS, long ldr, double *X, long ldx,
           const gb_bcg_args *args, void *work, size_t work_bytes);
size_t gb_bcg_work_bytes(int n, int k, int precision);
/* R[:, c] = s_c (lam_c BX[:, bi[c]] - AX[:, ai[c]]), s_c = 1 if |lam_c| <= 1 else 1 / lam_c */
int gb_w_residual(gcge_gpu_ctx *ctx, int n, int k, const double *AX, long ldax, const int *ai, const double *BX,
                  long ldbx, const int *bi, const double *lam, double *R, long ldr);

/* ------------------------------------------------------------ gb_dense.cu */
/* C = alpha op(A) op(B) + beta C, small column-major matrices on the device */
int gb_small_gemm(gcge_gpu_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                  const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);
/* Cholesky with deflation of a k x k Gram matrix G (column-major, ld ldg):
 * T (k x k, ld k) receives the coefficients that map the k input columns to the
 * kept, orthonormalised columns packed at the front; *kept_dev the kept count. */
int gb_chol_deflate(gcge_gpu_ctx *ctx, int k, const double *G, int ldg, double *T, int *kept_dev,
                    double zero_tol, double rel_tol, double *work);
/* partial symmetric eigensolve: eigenpairs il..iu (1-based, ascending) of the
 * m x m symmetric matrix H (column-major, ld ldh, full storage);
 * eval[0:iu-il+1], Z (m x (iu-il+1), ld ldz). work: gb_syevx_work_doubles(m). */
size_t gb_syevx_work_doubles(int m);
int gb_syevx(gcge_gpu_ctx *ctx, int m, const double *H, int ldh, int il, int iu, double *eval,
             double *Z, int ldz, double *work, int *info_dev);
/* the same with an estimate of each wanted eigenvalue (device array of iu-il+1
 * values, the previous Rayleigh-Ritz step's; may alias eval) that narrows the
 * bisection's starting intervals */
int gb_syevx_guess(gcge_gpu_ctx *ctx, int m, const double *H, int ldh, int il, int iu, double *eval, double *Z,
                   int ldz, double *work, int *info_dev, const double *guess);
/* small helpers used by the solver */
int gb_set_zero(gcge_gpu_ctx *ctx, double *a, size_t count);
int gb_copy_d(gcge_gpu_ctx *ctx, double *dst, const double *src, size_t count);
int gb_set_diag_from(gcge_gpu_ctx *ctx, double *H, int ldh, int count, const double *vals);
/* nu[i] = v[i], v[i] = -1 / v[i] for i < count (A-orthogonal Rayleigh-Ritz) */
int gb_neg_recip(gcge_gpu_ctx *ctx, int count, double *v, double *nu);
int gb_symmetrize_from_upper(gcge_gpu_ctx *ctx, double *H, int ldh, int m);
/* soft locking of the first s Ritz vectors: H's W columns (from w0) decoupled from
 * them, C[:, 0:s] = identity columns, C[0:s, s:iu] = 0 */
int gb_soft_lock(gcge_gpu_ctx *ctx, double *H, int ldh, int m, int w0, int s, double *C, int ldc, int iu);
int gb_copy_block(gcge_gpu_ctx *ctx, int rows, int cols, const double *src, int lds, double *dst, int ldd);
/* P-coefficient assembly of ComputeP (src/gcge_xpw.c:325-330) */
int gb_p_coef_assemble(gcge_gpu_ctx *ctx, double *coef, int ldc, int p_start, int p_ncols, int xx_nrows,
                       const int *unlock_dev);

#ifdef __cplusplus
}
#endif
#endif
