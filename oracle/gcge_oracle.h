/*
 * gcge_oracle.h -- CPU restatement of GCGE-1.0's CSR eigensolver path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle). Nothing in the product links this
 * library; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it, as the checker.
 *
 * Every function restates the reference algorithm step for step (same
 * operation order, same parameter defaults, same quirks) so that, given the
 * same initial vectors, its iterates agree with the compiled reference to
 * rounding level. Citations are file:line inside the GCGE-1.0 project.
 *
 * Multivectors passed across this interface are column-major n x k arrays
 * with leading dimension n.
 */
#ifndef GCGE_ORACLE_H
#define GCGE_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Solver parameters; defaults follow GCGE_PARA_Create (src/gcge_para.c:25-99). */
typedef struct {
    int    nev;                 /* number of wanted eigenpairs                          */
    int    block_size;          /* 0 -> nev (src/gcge_para.c:364-368)                   */
    int    ev_max_it;           /* outer GCG iterations (default 30)                    */
    int    cg_max_it;           /* block-CG iterations (default 20)                     */
    int    max_reorth_time;     /* default 3                                            */
    int    dirichlet_boundary;  /* zero Dirichlet rows of the initial X (csr app :130)  */
    int    given_init_evec;     /* 1: evec holds the initial vectors on entry           */
    double ev_tol;              /* default 1e-8                                         */
    double cg_rate;             /* default 1e-2                                         */
    double orth_zero_tol;       /* default 1e-16 (+DBL_EPSILON at setup)                */
    double reorth_tol;          /* default 0.75                                         */
    double scbgs_reorth_tol;    /* default 1e-16 (+DBL_EPSILON at setup)                */
    double criterion_tol;       /* default 1e-6                                         */
    char   conv_type[4];        /* "R" relative, "A" absolute, "O" omega-norm,
                                   "BR": ||Ax - lambda Bx|| / (|lambda| ||Bx||)         */
    int    init_rng;            /* 0: libc rand() after srand(seed) (the reference's),
                                   1: counter-hash uniform [0,1) shared with the GPU    */
    unsigned long long seed;
    int    print_level;         /* 0 silent, 1 per-iteration line                       */
    char   w_orth_type[8];      /* GCGE's w_orth_type ("" = "multi"; src/gcge_eigsol.c:448-472):
                                   every variant is restated (multi, bgs, cbgs, scbgs,
                                   the fallback GCGE_Orthonormalization)                */
    char   orth_type[4];        /* reference build only: "A" orthonormalises in the A inner
                                   product (src/gcge_eigsol.c:100-113); "" = "B" */
    int    opt_rr_eig_partly;   /* soft locking in the Rayleigh-Ritz eigensolve
                                   (src/gcge_rayleighritz.c:364-400), restated too      */
} gcge_oracle_params;

typedef struct {
    int    num_iter;
    int    num_unlock;
    double max_res, min_res, sum_res;
    double wall_s;              /* wall time of the solve (CLOCK_MONOTONIC)            */
    int    status;              /* 0 ok                                                 */
} gcge_oracle_stats;

void gcge_oracle_default_params(gcge_oracle_params *p);

/* Full GCGE solve, GCGE_Solve (src/gcge_eigsol.c:65-542) on the CSR backend.
 * B may be NULL (B = I). eval[nev], evec[n*nev] (column-major) are outputs
 * (evec is also the input when given_init_evec = 1). Returns 0 on success. */
int gcge_oracle_solve(int n,
                      const int *A_rp, const int *A_ci, const double *A_v,
                      const int *B_rp, const int *B_ci, const double *B_v,
                      const gcge_oracle_params *p,
                      double *eval, double *evec, gcge_oracle_stats *st);

/* The same GCGE_Solve restatement over a caller's GCGE_OPS table (layout
 * GCGE_GPU_OPS_LAYOUT, include/gcge_gb300_ops.h, member for member the
 * reference's GCGE_OPS, src/gcge_ops.h:29-215): GCGE's solver core driving
 * another backend through the table alone. A, B (B may be NULL) are the
 * table's matrix handles, n their order; evec is the eigenvector multivector
 * (nev handles, made by the table's MultiVecCreateByMat, as
 * GCGE_CSR_Solver_Init does, app/csr/gcge_app_csr.c:104-112); eval[nev] gets
 * the eigenvalues. Every n-sized operation goes through the table; the small
 * dense work stays on the host as the reference's defaults
 * (src/gcge_ops.c:573-604), except DenseMatEigenSolver, taken from the table.
 * The table's MultiVecSwap must exchange column data (as the GB300 table
 * does) or evec may end up holding workspace handles freed at exit. The
 * initial vectors come from the table's MultiVecSetRandomValue. Returns 0 on
 * success, 1 when the table lacks a member the solve needs. */
int gcge_oracle_solve_table(void *ops_table, void *A, void *B, int n, const gcge_oracle_params *p,
                            double *eval, void **evec, gcge_oracle_stats *st);

/* helpers for the table-driven solve: the table size, a copy of the host CSR
 * table (the reference's GCGE_CSR_SetOps plus defaults), a host CSR handle,
 * multivectors made and destroyed through a table, host columns read out */
size_t gcge_oracle_table_bytes(void);
void gcge_oracle_host_table(void *table);
void *gcge_oracle_csr_handle(int n, const int *rp, const int *ci, const double *v);
void gcge_oracle_csr_handle_free(void *A);
int  gcge_oracle_table_mv_create(void *table, void *mat, int k, void ***mv);
void gcge_oracle_table_mv_destroy(void *table, void ***mv, int k);
void gcge_oracle_host_mv_read(void **mv, int k, int n, double *out);

/* ---- double-double checker arithmetic (finite-difference checks) ----
 * Rayleigh quotient (x^T A x)/(x^T x), residual A x - theta x, x += d and
 * (sum w_i x_i^2, sum x_i^2), with x = xh + xl held as a double-double vector
 * (xl may be NULL) and every sum formed by error-free transformations. */
void gcge_oracle_dd_rayleigh(int n, const int *rp, const int *ci, const double *v, const double *xh,
                             const double *xl, double *out);
void gcge_oracle_dd_residual(int n, const int *rp, const int *ci, const double *v, const double *xh,
                             const double *xl, double th_hi, double th_lo, double *r);
void gcge_oracle_dd_add_vec(int n, double *xh, double *xl, const double *d);
void gcge_oracle_dd_weighted_sq(int n, const double *w, const double *xh, const double *xl, double *out);

/* ---- single operations, for per-kernel parity ---- */

/* y = A x  (app/csr/gcge_app_csr.c:297-323) */
void gcge_oracle_csr_matvec(int n, const int *rp, const int *ci, const double *v,
                            const double *x, double *y);
/* Y[:, j] = A X[:, j] for k columns (src/gcge_ops.c:115-129) */
void gcge_oracle_csr_matmultivec(int n, int k, const int *rp, const int *ci, const double *v,
                                 const double *X, double *Y);
/* y = a x + b y with the backend's special cases (app/csr/gcge_app_csr.c:330-365) */
void gcge_oracle_vec_axpby(int n, double a, const double *x, double b, double *y);
/* Y[:, j] = sum_i X[:, i] * coef[j*lda + i]  (src/gcge_ops.c:163-193) */
void gcge_oracle_multivec_lincomb(int n, int nx, int ny, const double *X, double *Y,
                                  const double *coef, int lda);
/* a = V^T W, "sym" fills the upper triangle and mirrors (src/gcge_ops.c:198-281) */
void gcge_oracle_multivec_innerprod(int n, int nv, int nw, const double *V, const double *W,
                                    double *a, int lda, int sym);
/* Block CG on A W = RHS, GCGE_BCG (src/gcge_cg.c:137-302). RHS is overwritten by
 * the residual, W (n x k) holds the initial guess on entry and the solution on exit. */
void gcge_oracle_bcg(int n, int k, const int *rp, const int *ci, const double *v,
                     double *RHS, double *W, int cg_max_it, double cg_rate);
/* B-orthonormalise V[:, start:end) against V[:, 0:start) and itself with the default
 * "multi" method, GCGE_StableMultiOrthonormalization (src/gcge_orthogonal.c:1833-1877).
 * B may be NULL. Returns the new end (zero vectors are moved past it). */
int gcge_oracle_stable_multi_orth(int n, int ncols, double *V, int start, int end,
                                  const int *B_rp, const int *B_ci, const double *B_v,
                                  int max_reorth_time, double orth_zero_tol, double scbgs_reorth_tol);

/* Uniform [0,1) counter-hash value used for initial vectors when init_rng = 1;
 * the GPU solver draws from the same function. */
double gcge_oracle_hash_uniform(unsigned long long seed, unsigned long long index);

#ifdef __cplusplus
}
#endif
#endif
