/*
 * gcge_gb300_ops.h -- GCGE_OPS plug-in table backed by the GB300 library.
 *
 * GCGE's solver core talks to its backend only through the GCGE_OPS table of
 * function pointers (src/gcge_ops.h:29-215). GCGE_GPU_SetOps fills that table
 * with device implementations so that the existing GCGE_SOLVER_* / GCGE_PARA /
 * workspace calls run unchanged on one GPU:
 *
 *     GCGE_SOLVER *s;  GCGE_SOLVER_Create(&s);
 *     GCGE_GPU_SetOps(ctx, s->ops);          (instead of GCGE_CSR_SetOps)
 *     ... GCGE_SOLVER_SetMatA(s, A_gpu); GCGE_SOLVER_Setup(s); GCGE_SOLVER_Solve(s);
 *
 * GCGE_GPU_OPS_LAYOUT restates the member order and types of GCGE_OPS with
 * GCGE_DOUBLE = double and GCGE_INT = int (src/gcge_config.h:23-24), so the
 * table can be filled without including the reference headers; the two layouts
 * must stay identical member for member.
 *
 * Handles placed in the table:
 *  - matrix (void *): gcge_gpu_mat * from GCGE_GPU_MatCreate;
 *  - vector (void *): a column of a device multivector (a standalone vector is
 *    a one-column multivector);
 *  - multivector (void **): an array of vector handles that all refer to
 *    consecutive columns of one row-major device block. MultiVecSwap exchanges
 *    column data (not handles), so this invariant holds for the whole solve.
 *
 * Filled members: every vector and multivector member, GetVecFromMultiVec /
 * RestoreVecForMultiVec, SetDirichletBoundary and DenseMatEigenSolver (the
 * dsyevx-signature eigensolve, run on the device). The small dense BLAS members
 * (DenseMatDotDenseMat, DenseSymMatDotDenseMat, Array*) are left as they are,
 * so GCGE_OPS_Setup (src/gcge_ops.c:573-604) installs its host defaults.
 * Orthonormalization is left as it is; LinearSolver is left unset unless
 * GCGE_GPU_OpsSetLinearSolver installs a device solver there.
 *
 * The members return void, as in the reference; failures are recorded on the
 * context and read with GCGE_GPU_GetLastError after GCGE_SOLVER_Solve.
 * One table is bound to one context at a time (the reference core is itself
 * single-threaded and not re-entrant).
 */
#ifndef GCGE_GB300_OPS_H
#define GCGE_GB300_OPS_H

#include "gcge_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GCGE_GPU_OPS_LAYOUT_ {
    void (*VecSetRandomValue)(void *vec);
    void (*MatDotVec)(void *Matrix, void *x, void *r);
    void (*VecAxpby)(double a, void *x, double b, void *y);
    void (*VecInnerProd)(void *x, void *y, double *value_ip);
    void (*VecLocalInnerProd)(void *x, void *y, double *value_ip);
    void (*VecCreateByVec)(void **des_vec, void *src_vec);
    void (*VecCreateByMat)(void **vec, void *mat);
    void (*VecDestroy)(void **vec);
    void (*LinearSolver)(void *Matrix, void *b, void *x, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void *linear_solver_workspace;
    void (*Orthonormalization)(void **V, int start, int *end, void *B, double orth_zero_tol, void **work);
    void (*DenseMatCreate)(void **densemat, int nrows, int ncols);
    void (*DenseMatDestroy)(void **mat);
    void (*MultiVecCreateByVec)(void ***multi_vec, int n_vec, void *vec, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecCreateByMat)(void ***multi_vec, int n_vec, void *mat, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecCreateByMultiVec)(void ***multi_vec, int n_vec, void **init_vec,
                                     struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecDestroy)(void ***MultiVec, int n_vec, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecSetRandomValue)(void **multi_vec, int start, int n_vec, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MatDotMultiVec)(void *mat, void **x, void **y, int *start, int *end, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecAxpby)(double a, void **x, double b, void **y, int *start, int *end,
                          struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecAxpbyColumn)(double a, void **x, int col_x, double b, void **y, int col_y,
                                struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecLinearComb)(void **x, void **y, int *start, int *end, double *a, int lda, void *dmat,
                               int lddmat, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecInnerProd)(void **V, void **W, double *a, char *is_sym, int *start, int *end, int lda,
                              struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecSwap)(void **V_1, void **V_2, int *start, int *end, struct GCGE_GPU_OPS_LAYOUT_ *ops);
    void (*MultiVecPrint)(void **x, int n);
    void (*GetVecFromMultiVec)(void **V, int j, void **x);
    void (*RestoreVecForMultiVec)(void **V, int j, void **x);
    void (*SetDirichletBoundary)(void **Vecs, int nev, void *A, void *B);
    void (*DenseMatEigenSolver)(char *jobz, char *range, char *uplo, int *nrows, double *a, int *lda,
                                double *vl, double *vu, int *il, int *iu, double *abstol, int *nev,
                                double *eval, double *evec, int *lde, int *isuppz, double *work, int *lwork,
                                int *iwork, int *liwork, int *ifail, int *info);
    void (*DenseMatDotDenseMat)(char *transa, char *transb, int *nrows, int *ncols, int *mid, double *alpha,
                                double *a, int *lda, double *b, int *ldb, double *beta, double *c, int *ldc);
    void (*DenseSymMatDotDenseMat)(char *side, char *uplo, int *nrows, int *ncols, double *alpha, double *a,
                                   int *lda, double *b, int *ldb, double *beta, double *c, int *ldc);
    double (*ArrayDotArray)(double *x, double *y, int length);
    double (*ArrayNorm)(double *x, int length);
    void (*ArrayAXPBY)(double a, double *x, double b, double *y, int length);
    void (*ArrayCopy)(double *x, double *y, int length);
    void (*ArrayScale)(double alpha, double *a, int length);
} GCGE_GPU_OPS_LAYOUT;

/* Fill the device members of a GCGE_OPS table (passed as void * so that this
 * header does not depend on the reference's) and bind it to ctx; replaces
 * GCGE_CSR_SetOps (app/csr/gcge_app_csr.c:70-84). */
int GCGE_GPU_SetOps(gcge_gpu_ctx *ctx, void *gcge_ops);

/* Seed of the counter-hash generator behind VecSetRandomValue and
 * MultiVecSetRandomValue (the reference's CSR backend draws from libc rand(),
 * app/csr/gcge_app_csr.c:284-294). */
void GCGE_GPU_OpsSeed(unsigned long long seed);

/* Device multivector behind a table multivector handle (void **), with the
 * column its first handle refers to. */
int GCGE_GPU_OpsMultiVecBlock(void **multi_vec, gcge_gpu_mv **block, int *first_col);

/* Install a device linear solver in the table's LinearSolver member, which the
 * reference calls once per W column in place of its block CG
 * (src/gcge_xpw.c:177-191): kind 0 removes it (the reference's GCGE_BCG runs),
 * kind 1 installs Jacobi-preconditioned CG (z = diag(A)^-1 r) run from the given
 * x to ||r||_z <= rate ||r0||_z or max_it iterations (b is left unchanged). The
 * reference's hook signature (A, b, x, ops) carries no parameters, so max_it and
 * rate are held by the library for every table. No counterpart in the reference
 * beyond the hook itself (its users install HYPRE solvers there). */
int GCGE_GPU_OpsSetLinearSolver(void *gcge_ops, int kind, int max_it, double rate);

#ifdef __cplusplus
}
#endif
#endif
