/*
 * gcge_gb300.h -- C ABI of the GB300-native GCGE CSR eigensolver path.
 *
 * One process, one GPU (sm_103a). All entry points are plain C: opaque handles,
 * host pointers and sizes, an int status (GCGE_GPU_OK = 0 on success). No CPU
 * fallback exists: without a usable CUDA device every call fails with
 * GCGE_GPU_ERR_CUDA.
 *
 * The entry points fall in four groups, each replacing a reference interface
 * (file:line inside the GCGE-1.0 project):
 *
 *  1. Device data.  GCGE_GPU_MatCreate uploads a CSR matrix in the reference's
 *     CSR_MAT layout (app/csr/gcge_app_csr.h:27-40); GCGE_GPU_MultiVecCreate
 *     allocates a multivector (the role of ops->MultiVecCreateByMat,
 *     src/gcge_ops.h:59). Multivectors live in HBM as row-major n x ncols
 *     blocks (each row of the block contiguous).
 *  2. Block operations with the semantics of the GCGE_OPS multivector members
 *     (src/gcge_ops.h:57-86): MatDotMultiVec, MultiVecAxpby, MultiVecLinearComb,
 *     MultiVecInnerProd, MultiVecSwap. Column ranges are half open
 *     [start[i], end[i]); index 0 refers to the first multivector argument,
 *     index 1 to the second; dense coefficient arrays are column major with an
 *     explicit leading dimension, as in the reference.
 *  3. The plug-in table. GCGE_GPU_SetOps fills a GCGE_OPS table
 *     (src/gcge_ops.h:29-215) with device implementations, so GCGE's own
 *     GCGE_SOLVER_* calls run on the GPU. See gcge_gb300_ops.h.
 *  4. The GPU-native solver. GCGE_GPU_Solve runs the whole GCG iteration of
 *     GCGE_Solve (src/gcge_eigsol.c:65-542) on the device with the GCGE_PARA
 *     parameters (src/gcge_para.h:41-103); GCGE_GPU_SolveHost does the same from
 *     host CSR arrays, the counterpart of GCGE_CSR_Solver_Init + GCGE_SOLVER_Solve
 *     (app/csr/gcge_app_csr.c:92-124, src/gcge_solver.c:98-101).
 */
#ifndef GCGE_GB300_H
#define GCGE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define GCGE_GPU_OK            0
#define GCGE_GPU_ERR_ARG       1   /* invalid argument (sizes, ranges, NULL)            */
#define GCGE_GPU_ERR_CUDA      2   /* CUDA runtime error (no device, launch failure)    */
#define GCGE_GPU_ERR_NOMEM     3   /* device allocation failed                          */
#define GCGE_GPU_ERR_CSR       4   /* malformed CSR (row pointers, column range)        */
#define GCGE_GPU_ERR_NONFINITE 5   /* NaN/Inf met in a reduction or the small eigensolve */
#define GCGE_GPU_ERR_BREAKDOWN 6   /* orthogonalisation lost every column               */
#define GCGE_GPU_ERR_EIGSOLVE  7   /* projected eigensolve did not converge             */
#define GCGE_GPU_ERR_TIMEOUT   8   /* a tensor-core kernel's bounded wait ran out       */
#define GCGE_GPU_ERR_IO        9   /* file missing, unreadable, truncated or not CSR    */

typedef struct gcge_gpu_ctx gcge_gpu_ctx;  /* device, stream, reduction scratch  */
typedef struct gcge_gpu_mat gcge_gpu_mat;  /* CSR matrix resident in HBM         */
typedef struct gcge_gpu_mv  gcge_gpu_mv;   /* row-major multivector in HBM       */

/* Context: binds a CUDA device and creates the stream every call is ordered on. */
int  GCGE_GPU_Init(int device, gcge_gpu_ctx **ctx);
int  GCGE_GPU_Finalize(gcge_gpu_ctx *ctx);
/* The first error any call on this context met (sticky), then cleared. The
 * GCGE_OPS table members return void as in the reference, so they record their
 * failures here. */
int  GCGE_GPU_GetLastError(gcge_gpu_ctx *ctx);
const char *GCGE_GPU_ErrorString(int status);
int  GCGE_GPU_Synchronize(gcge_gpu_ctx *ctx);

/* ---- 1. device data ---- */

/* Upload an n x n CSR matrix (RowPtr[n+1], KCol[nnz], Entries[nnz], as CSR_MAT,
 * app/csr/gcge_app_csr.h:27-40). keep_fp32 != 0 also keeps an FP32 copy of the
 * values for the mixed-precision inner solve, and lists the rows longer than 64
 * entries (one host pass over rowptr) for the FP32 product, which gives each of
 * them a block. The structure is checked on the device after the upload
 * (GCGE_GPU_ERR_CSR: rowptr[0] != 0, a decreasing row pointer or a column index
 * outside [0, n)). */
int  GCGE_GPU_MatCreate(gcge_gpu_ctx *ctx, int n, const int *rowptr, const int *col,
                        const double *val, int keep_fp32, gcge_gpu_mat **A);
/* Replace the values (same pattern); refreshes the FP32 copy if kept. */
int  GCGE_GPU_MatSetValues(gcge_gpu_mat *A, const double *val);
int  GCGE_GPU_MatDestroy(gcge_gpu_mat *A);
int  GCGE_GPU_MatGetSize(const gcge_gpu_mat *A, int *n, int *nnz);

/* CSR files (host only, no device needed). Text: the reference's format
 * (CSR_ReadMatFile, app/csr/gcge_app_csr.c:185-236): nrow, ncol, nnz, RowPtr[nrow+1],
 * KCol[nnz], Entries[nnz], white-space separated, 0-based; a failure returns a
 * status (GCGE_GPU_ERR_IO, GCGE_GPU_ERR_CSR) where the reference exits. Binary:
 * "GCGECSR\1", int32 nrow, int32 ncol, int64 nnz, then the three arrays (int32,
 * int32, float64), little endian. The readers allocate the arrays; release them
 * with GCGE_GPU_CSRFree. MatCreateFromFile reads either form (by the header) and
 * uploads it (square matrices), the reading part of GCGE_CSR_Solver_Init
 * (app/csr/gcge_app_csr.c:92-124). */
int  GCGE_GPU_CSRReadText(const char *path, int *nrow, int *ncol, int *nnz, int **rowptr, int **col,
                          double **val);
int  GCGE_GPU_CSRReadBinary(const char *path, int *nrow, int *ncol, int *nnz, int **rowptr, int **col,
                            double **val);
int  GCGE_GPU_CSRWriteBinary(const char *path, int nrow, int ncol, int nnz, const int *rowptr, const int *col,
                             const double *val);
void GCGE_GPU_CSRFree(int *rowptr, int *col, double *val);
int  GCGE_GPU_MatCreateFromFile(gcge_gpu_ctx *ctx, const char *path, int keep_fp32, gcge_gpu_mat **A);

int  GCGE_GPU_MultiVecCreate(gcge_gpu_ctx *ctx, int n, int ncols, gcge_gpu_mv **mv);
int  GCGE_GPU_MultiVecDestroy(gcge_gpu_mv *mv);
/* Host <-> device copies of columns [col0, col0+ncols); host arrays are column
 * major n x ncols (leading dimension n), the reference's vector-per-column view. */
int  GCGE_GPU_MultiVecUpload(gcge_gpu_mv *mv, int col0, int ncols, const double *host);
int  GCGE_GPU_MultiVecDownload(const gcge_gpu_mv *mv, int col0, int ncols, double *host);
/* Fill columns [start, start+nvec) with uniform [0,1) values of the counter hash
 * (seed, column*n + row); ops->MultiVecSetRandomValue, src/gcge_ops.h:66. */
int  GCGE_GPU_MultiVecSetRandomValue(gcge_gpu_mv *mv, int start, int nvec, unsigned long long seed);

/* Dense FP64 contractions (Gram products, linear combinations) either on the
 * bf16 tensor cores with an error-free digit splitting that keeps FP64 accuracy
 * (on = 1, the default) or on the FP64 pipe (on = 0). No counterpart in the
 * reference (its dense work is host BLAS). */
int  GCGE_GPU_SetTensorEmulation(gcge_gpu_ctx *ctx, int on);

/* Test hook for the failure path of the tensor-core kernels (no counterpart in
 * the reference). With on != 0, the next tensor-core launch on this context
 * (Gram or linear combination) has its MMA-issuing thread wait, before the first
 * stage, for an arrival that cannot come, so that its bounded wait (1 s of
 * %globaltimer) runs out: the CTAs take the timeout path (wait, bounded, for
 * their own copies in flight, free their TMEM, return), the context's device
 * error word is set, GCGE_GPU_Synchronize reports GCGE_GPU_ERR_TIMEOUT, and
 * later tensor-core launches on this context do no work. One-shot: the flag is
 * cleared by that launch. No fault, trap or endless wait is involved. */
int  GCGE_GPU_TestStallTensorWait(gcge_gpu_ctx *ctx, int on);

/* Sparse products Y = A X with two or more columns either in FP32-pair
 * arithmetic (on = 1: values as hi + lo floats, error-free products and sums on
 * the FP32 pipe, ~1e-14 of sum |a_ij x_j|; |x| >= 2^100 or non-finite X falls
 * back to FP64 inside the product) or on the FP64 pipe (on = 0, the default). A
 * solve with precision 2 switches it on for its own duration. No counterpart in
 * the reference. */
int  GCGE_GPU_SetPairSpMM(gcge_gpu_ctx *ctx, int on);

/* ---- 2. block operations (semantics of src/gcge_ops.c:115-300) ---- */

/* y(:, start[1]:end[1]) = A x(:, start[0]:end[0]); ops->MatDotMultiVec,
 * src/gcge_ops.h:67 (default loop src/gcge_ops.c:115-129). */
int  GCGE_GPU_MatDotMultiVec(const gcge_gpu_mat *A, const gcge_gpu_mv *x, gcge_gpu_mv *y,
                             const int *start, const int *end);
/* y(:, s1:e1) = a x(:, s0:e0) + b y(:, s1:e1), with CSR_VecAxpby's special cases
 * (a == 0: y = b y; b == 0: y = a x); ops->MultiVecAxpby, src/gcge_ops.h:69. */
int  GCGE_GPU_MultiVecAxpby(double a, const gcge_gpu_mv *x, double b, gcge_gpu_mv *y,
                            const int *start, const int *end);
/* y(:, s1:e1) = x(:, s0:e0) * a, a column major (e0-s0) x (e1-s1) host array with
 * leading dimension lda; ops->MultiVecLinearComb, src/gcge_ops.h:74. */
int  GCGE_GPU_MultiVecLinearComb(const gcge_gpu_mv *x, gcge_gpu_mv *y, const int *start,
                                 const int *end, const double *a, int lda);
/* a(0:e0-s0, 0:e1-s1) = V(:, s0:e0)^T W(:, s1:e1) into a host array with leading
 * dimension lda; is_sym "sym" computes the upper triangle and mirrors it.
 * ops->MultiVecInnerProd, src/gcge_ops.h:77 (src/gcge_ops.c:198-281). */
int  GCGE_GPU_MultiVecInnerProd(const gcge_gpu_mv *V, const gcge_gpu_mv *W, double *a,
                                const char *is_sym, const int *start, const int *end, int lda);
/* Exchange V1(:, s0:e0) and V2(:, s1:e1) (data, not handles); ops->MultiVecSwap,
 * src/gcge_ops.h:79. */
int  GCGE_GPU_MultiVecSwap(gcge_gpu_mv *V1, gcge_gpu_mv *V2, const int *start, const int *end);

/* Block CG on A W = RHS for k columns, GCGE_BCG (src/gcge_cg.c:137-302): W (initial
 * guess in, solution out) and RHS (overwritten by the residual) are the column
 * ranges [w_start, w_start+k) and [r_start, r_start+k). precision 0: FP64;
 * 1: FP32 vectors and FP32 matrix values with FP64-accumulated dot products
 * (requires keep_fp32 on A). */
int  GCGE_GPU_BCG(const gcge_gpu_mat *A, gcge_gpu_mv *RHS, int r_start, gcge_gpu_mv *W,
                  int w_start, int k, int cg_max_it, double cg_rate, int precision);

/* B-orthonormalise W(:, start:*end) against W(:, 0:start) (already B-orthonormal)
 * and itself: block projection passes, then Cholesky-QR twice with deflation of
 * dependent columns (kept columns are packed to the front, *end shrinks). Role of
 * GCGE_StableMultiOrthonormalization, src/gcge_orthogonal.c:1833-1877. B may be NULL. */
int  GCGE_GPU_Orthonormalize(gcge_gpu_mv *W, int start, int *end, const gcge_gpu_mat *B,
                             int max_reorth_time, double orth_zero_tol);
/* The same with the variant named as the reference's w_orth_type: "multi" (the
 * call above), "cbgs", "scbgs", or column-by-column Gram-Schmidt for any other
 * name ("bgs", "gs"). */
int  GCGE_GPU_OrthonormalizeType(gcge_gpu_mv *W, int start, int *end, const gcge_gpu_mat *B, int max_reorth_time,
                                 double orth_zero_tol, const char *w_orth_type);

/* ---- 4. GPU-native solver ---- */

/* GCGE_PARA members that drive the solve (src/gcge_para.h:41-103, defaults of
 * GCGE_PARA_Create src/gcge_para.c:25-99), plus precision and the seed of the
 * initial vectors. */
typedef struct {
    int    nev;               /* wanted eigenpairs                                   */
    int    block_size;        /* 0 -> nev                                             */
    int    ev_max_it;         /* 30                                                   */
    int    cg_max_it;         /* 20                                                   */
    int    max_reorth_time;   /* 3                                                    */
    int    dirichlet_boundary;/* zero Dirichlet rows of the initial X                  */
    int    given_init_evec;   /* 1: evec holds the initial vectors                    */
    double ev_tol;            /* 1e-8                                                 */
    double cg_rate;           /* 1e-2                                                 */
    double orth_zero_tol;     /* 1e-16 (+DBL_EPSILON)                                 */
    char   conv_type[4];      /* "R", "A", "O" as the reference; "BR":
                                 ||Ax - lambda Bx|| / (|lambda| ||Bx||)               */
    int    precision;         /* 0 plain FP64; 1 mixed (FP32 inner block CG);
                                 2 mixed, and the outer sparse products (A W, B W,
                                 A X, B X) in FP32-pair arithmetic (48-bit
                                 significand, ~1e-14 of sum |a_ij x_j|)              */
    unsigned long long seed;  /* counter-hash seed of the initial vectors             */
    int    print_level;       /* 0 silent; 1 one line per iteration (reference format)*/
    int    precond;           /* inner block CG: 0 plain (GCGE_BCG, the default);
                                 1 Jacobi-preconditioned (z = diag(A)^-1 r, rho = r.z),
                                 the role of a user linear solver installed in
                                 ops->LinearSolver (src/gcge_xpw.c:177-191)          */
    char   w_orth_type[8];    /* W orthonormalisation (src/gcge_eigsol.c:448-472):
                                 "multi" (default: block projection + Cholesky-QR
                                 twice), "cbgs" / "scbgs" (block projections, then
                                 the eigenvectors of W^T B W, once / twice), any
                                 other name column-by-column Gram-Schmidt          */
    int    opt_rr_eig_partly; /* 1: soft locking (src/gcge_rayleighritz.c:364-400):
                                 the converged leading Ritz pairs before the first
                                 unconverged one (and its near-multiples) are kept,
                                 only the trailing projected block is solved      */
    double multi_tol_for_lock;/* 1e-6: relative gap under which an earlier
                                 eigenvalue is taken as a multiple of it          */
    char   orth_type[4];      /* "B" (default): the basis is B-orthonormal and the
                                 Rayleigh-Ritz matrix is V^T A V; "A": the basis is
                                 A-orthonormal (A must be positive definite), the
                                 projected matrix is V^T B V, whose largest
                                 eigenvalues mu give lambda = 1/mu (the role of
                                 orth_type "A", src/gcge_eigsol.c:100-113, with
                                 GCGE_SortEigenpairs, src/gcge_rayleighritz.c:581-617);
                                 the eigenvectors are returned A-orthonormal      */
} gcge_gpu_params;

typedef struct {
    int    num_iter;          /* outer GCG iterations (para->num_iter)                 */
    int    num_unlock;        /* eigenpairs still above ev_tol                         */
    double max_res, min_res, sum_res;
    double res[8];            /* unused, reserved                                      */
    double solve_ms;          /* device time of the solve (CUDA events)                */
    double phase_ms[9];       /* GCGE_PART_TIME slots (src/gcge_statistics.h:23-33):
                                 x_axpy, x_orth, p_axpy, p_orth, w_line, w_orth,
                                 rr_mat, rr_eigen, conv                                */
    long long kernel_launches;/* kernels this library launched during the solve        */
    long long spmm_calls;     /* CSR SpMM launches (FP64 + FP32)                       */
} gcge_gpu_stats;

void GCGE_GPU_ParamsDefault(gcge_gpu_params *p);

/* Solve A x = lambda B x for the nev smallest eigenpairs with device-resident A,
 * B (B may be NULL: B = I). eval: host array [nev]; evec: multivector with at
 * least nev columns (read when given_init_evec = 1, holds the eigenvectors on exit). */
int  GCGE_GPU_Solve(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B,
                    const gcge_gpu_params *p, double *eval, gcge_gpu_mv *evec,
                    gcge_gpu_stats *stats);

/* Host-buffer entry: uploads the CSR arrays, solves, downloads eval[nev] and
 * evec (column major n x nev, leading dimension n), frees the device copies. */
int  GCGE_GPU_SolveHost(gcge_gpu_ctx *ctx, int n,
                        const int *A_rowptr, const int *A_col, const double *A_val,
                        const int *B_rowptr, const int *B_col, const double *B_val,
                        const gcge_gpu_params *p, double *eval, double *evec,
                        gcge_gpu_stats *stats);

/* Number of this library's kernel launches on the context so far (a counter the
 * host wrappers increment at every launch). Instrumentation with no counterpart
 * in the reference. */
long long GCGE_GPU_LaunchCount(const gcge_gpu_ctx *ctx);

/* Profiling mode (instrumentation, no counterpart in the reference): while on,
 * every launch of the hot kernels is bracketed by CUDA events on the context's
 * stream and attributed to a class with its algorithmic bytes and flops.
 * Classes, in order: 0 CSR SpMM FP64, 1 CSR SpMM FP32, 2 Gram V^T W,
 * 3 linear combination X*C, 4 block-CG vector updates and dots, 5 AXPBY/copies,
 * 6 small dense GEMM, 7 small dense eigensolve, 8 per-column reductions,
 * 9 CSR SpMM in FP32-pair arithmetic.
 * ProfileRead fills up to nclass entries of each non-NULL array and returns
 * the number of classes (reset != 0 zeroes the totals afterwards). */
int  GCGE_GPU_ProfileEnable(gcge_gpu_ctx *ctx, int on);
int  GCGE_GPU_ProfileRead(gcge_gpu_ctx *ctx, int nclass, double *ms, long long *launches,
                          double *bytes, double *flops, int reset);

/* ---- 5. differentiation (adjoint kernels; no counterpart in the reference) ----
 *
 * Gradients of a function of computed eigenpairs with respect to the stored
 * entries of A and B. Each stored entry (i, j) is one independent variable (a
 * symmetric perturbation of an off-diagonal pair is the sum of the gradients of
 * the two stored entries). For a B-orthonormal eigenpair (lambda, x):
 *   d lambda / d A_ij = x_i x_j,  d lambda / d B_ij = -lambda x_i x_j;
 * for a function L of a simple eigenvector x with g = dL/dx and mu from
 * GCGE_GPU_EigvecAdjoint:
 *   dL / d A_ij = -mu_i x_j,  dL / d B_ij = lambda mu_i x_j - (g^T x / 2) x_i x_j. */

/* grad[e] = sum_t scale[t] U(i, u0+t) V(j, v0+t) over t < r for every stored
 * entry e = (i, j) of M, in M's CSR order (accumulate != 0: added to grad).
 * grad: host array of nnz(M) doubles; scale: host array of r doubles;
 * r <= 768. */
int  GCGE_GPU_PatternGrad(const gcge_gpu_mat *M, const gcge_gpu_mv *U, int u0, const gcge_gpu_mv *V,
                          int v0, int r, const double *scale, int accumulate, double *grad);

/* mu (column mu_col of MU) solving (A - lambda_k B) mu = (I - B x_k x_k^T) g with
 * x_k^T B mu = 0, for the eigenpair (lambda_k, x_k) = (eval[k], X(:, k)) of the
 * B-orthonormal eigenvectors X(:, 0:m) (eval: host array of m values; B may be
 * NULL: B = I) and g = column g_col of G. The components along the other x_j are
 * x_j (x_j^T g) / (lambda_j - lambda_k), except inside k's cluster
 * (|lambda_j - lambda_k| <= cluster_tol |lambda_k|, left at zero); the rest
 * solves the shifted system on the B-complement of X(:, 0:m), where it is
 * positive definite when lambda_k is below the first eigenvalue not in X, by
 * FP64 conjugate gradients to relative residual tol in at most max_it
 * iterations (iters, if not NULL, returns the count). */
int  GCGE_GPU_EigvecAdjoint(const gcge_gpu_mat *A, const gcge_gpu_mat *B, const gcge_gpu_mv *X, int m,
                            const double *eval, int k, const gcge_gpu_mv *G, int g_col, gcge_gpu_mv *MU,
                            int mu_col, double cluster_tol, double tol, int max_it, int *iters);

/* ---- allocation-free Gram product (no counterpart in the reference) ----
 *
 * For callers that own all device memory through their own pool or arena and
 * may not call cudaMalloc / cudaFree (those calls can synchronise the device and
 * would take memory the pool has already claimed). Computes the Gram block of
 * GCGE_GPU_MultiVecInnerProd, a(0:k1, 0:k2) = V^T W ("sym": upper triangle
 * computed and mirrored), on caller memory and allocates nothing:
 *   V, W   device pointers to row-major blocks, element (r, c) at V[r*ldv + c]
 *          (the multivector layout of this library), n rows, k1 / k2 columns;
 *   a      device pointer, column major with leading dimension lda >= k1;
 *   stream a cudaStream_t (NULL: the default stream); the call is asynchronous.
 * Partial sums go to a fixed 8 MiB device array inside the library (held by
 * every GPU that loads it, until exit), so k1*k2 may be at most 262,144.
 * Larger sizes are rejected with GCGE_GPU_ERR_ARG. The first call on a device
 * looks up the array's device address with that device current; make that
 * first call before any stream capture. All calls share the array and it keeps
 * the last call's contents; calls that overlap on the GPU race on it. */
int  GCGE_GPU_InnerProdNoAlloc(int n, int k1, int k2, const double *V, long ldv, const double *W,
                               long ldw, double *a, int lda, int sym, void *stream);

#ifdef __cplusplus
}
#endif
#endif
