/*
 * gcge_oracle.c -- CPU restatement of GCGE-1.0's CSR eigensolver path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
 * product library.
 *
 * The reference keeps multivectors as arrays of independent column pointers
 * and exchanges columns by swapping pointers; this restatement does the same
 * (mv_t below) so that every phase of GCGE_Solve can be followed one to one.
 * Dense small-matrix work goes to LAPACK/BLAS exactly where the reference
 * calls it (dsyevx, dgemm, dsymm, ddot, dnrm2, dscal); they are taken from
 * SciPy's bundled OpenBLAS (symbols with the scipy_ prefix), the same library
 * the reference build in oracle/_ref links.
 */
#define _POSIX_C_SOURCE 199309L
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gcge_oracle.h"
#include "gcge_gb300_ops.h"

/* ------------------------------------------------------------------ LAPACK */
extern void scipy_dsyevx_(char *jobz, char *range, char *uplo, int *n, double *a, int *lda,
                          double *vl, double *vu, int *il, int *iu, double *abstol, int *m,
                          double *w, double *z, int *ldz, double *work, int *lwork,
                          int *iwork, int *ifail, int *info);
extern void scipy_dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha,
                         double *a, int *lda, double *b, int *ldb, double *beta,
                         double *c, int *ldc);
extern void scipy_dsymm_(char *side, char *uplo, int *m, int *n, double *alpha, double *a,
                         int *lda, double *b, int *ldb, double *beta, double *c, int *ldc);
extern double scipy_ddot_(int *n, double *x, int *incx, double *y, int *incy);
extern double scipy_dnrm2_(int *n, double *x, int *incx);
extern void scipy_dscal_(int *n, double *a, double *x, int *incx);

static double arr_dot(double *x, double *y, int n) { int one = 1; return scipy_ddot_(&n, x, &one, y, &one); }
static double arr_nrm2(double *x, int n) { int one = 1; return scipy_dnrm2_(&n, x, &one); }
static void arr_scal(double a, double *x, int n) { int one = 1; scipy_dscal_(&n, &a, x, &one); }
static void dgemm(char ta, char tb, int m, int n, int k, double alpha, double *a, int lda,
                  double *b, int ldb, double beta, double *c, int ldc)
{
    scipy_dgemm_(&ta, &tb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
}

/* --------------------------------------------------------------- CSR ops */
/* Every n-sized operation of the restatement goes through a table with the
 * GCGE_OPS layout (src/gcge_ops.h:29-215), as the reference's solver core does.
 * The default table below is the CSR backend of the reference (host arrays,
 * app/csr/gcge_app_csr.c:70-84, with the multivector defaults of
 * src/gcge_ops.c:115-300); gcge_oracle_solve_table runs the same restatement
 * over a caller's table (GCGE's core driving another backend). */
typedef GCGE_GPU_OPS_LAYOUT ops_t;
static ops_t *T;                  /* the table the current call goes through */

typedef struct { int n; const int *rp, *ci; const double *v; } csr_t;
/* CSR_VEC, app/csr/gcge_app_csr.h:42-46: a size and its entries */
typedef struct { int size; double *e; } hvec_t;
static double *hcol(void *v) { return ((hvec_t *)v)->e; }

/* app/csr/gcge_app_csr.c:297-323: zero y, then accumulate row by row */
static void h_matvec(void *mat, void *xv, void *yv)
{
    const csr_t *A = (const csr_t *)mat;
    const double *x = hcol(xv);
    double *y = hcol(yv);
    memset(y, 0, (size_t)A->n * sizeof(double));
    for (int i = 0; i < A->n; ++i)
        for (int j = A->rp[i]; j < A->rp[i + 1]; ++j)
            y[i] += A->v[j] * x[A->ci[j]];
}

/* app/csr/gcge_app_csr.c:330-365: y = a x + b y with its three special cases */
static void h_axpby(double a, void *xv, double b, void *yv)
{
    const int n = ((hvec_t *)yv)->size;
    const double *x = hcol(xv);
    double *y = hcol(yv);
    if (a == 0.0) {
        for (int i = 0; i < n; ++i) y[i] = b * y[i];
    } else if (b == 0.0) {
        if (a == 1.0) for (int i = 0; i < n; ++i) y[i] = x[i];
        else          for (int i = 0; i < n; ++i) y[i] = a * x[i];
    } else {
        for (int i = 0; i < n; ++i) y[i] = a * x[i] + b * y[i];
    }
}

/* app/csr/gcge_app_csr.c:368-378 */
static void h_dot(void *xv, void *yv, double *value)
{
    const int n = ((hvec_t *)xv)->size;
    const double *x = hcol(xv), *y = hcol(yv);
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[i] * y[i];
    *value = s;
}

/* the operations the restatement uses, each one table call */
static void csr_mv(void *A, void *x, void *y) { T->MatDotVec(A, x, y); }
static void vaxpby(double a, void *x, double b, void *y) { T->VecAxpby(a, x, b, y); }
static double vdot(void *x, void *y)
{
    double v = 0.0;
    T->VecInnerProd(x, y, &v);
    return v;
}

/* counter hash shared with the GPU solver's initial vectors (splitmix64 finaliser) */
double gcge_oracle_hash_uniform(unsigned long long seed, unsigned long long index)
{
    unsigned long long z = seed ^ (index * 0xD1B54A32D192ED03ULL);
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* ----------------------------------------------------------- multivector */
/* An ordered set of column handles; the reference's void** multivector. */
typedef struct { int n, k; void **c; hvec_t *vecs; double *store; } mv_t;

/* host columns over caller storage (base == NULL: owned, zeroed) */
static void h_mv_make(mv_t *m, int n, int k, double *base)
{
    m->n = n; m->k = k;
    m->store = base ? NULL : (double *)calloc((size_t)n * (k > 0 ? k : 1), sizeof(double));
    m->vecs = (hvec_t *)malloc(sizeof(hvec_t) * (k > 0 ? k : 1));
    m->c = (void **)malloc(sizeof(void *) * (k > 0 ? k : 1));
    for (int j = 0; j < k; ++j) {
        m->vecs[j].size = n;
        m->vecs[j].e = (base ? base : m->store) + (size_t)j * n;
        m->c[j] = &m->vecs[j];
    }
}
static void h_mv_free(mv_t *m)
{
    free(m->store); free(m->vecs); free(m->c);
    m->store = NULL; m->vecs = NULL; m->c = NULL;
}

/* the restatement's workspace: GCGE_WORKSPACE_Setup creates it through
 * ops->MultiVecCreateByMat (src/gcge_workspace.c:76-78) */
static int g_host;   /* 1: the current call runs on the host table */
static void mv_alloc(mv_t *m, void *mat, int n, int k)
{
    if (g_host) { h_mv_make(m, n, k, NULL); return; }
    m->n = n; m->k = k; m->vecs = NULL; m->store = NULL; m->c = NULL;
    T->MultiVecCreateByMat(&m->c, k, mat, T);
}
static void mv_free(mv_t *m)
{
    if (g_host) { h_mv_free(m); return; }
    if (m->c) T->MultiVecDestroy(&m->c, m->k, T);
    m->c = NULL;
}

/* src/gcge_ops.c:115-129 */
static void h_mv_matdot(void *A, void **x, void **y, int *s, int *e, ops_t *ops)
{
    for (int i = 0; i < e[0] - s[0]; ++i) ops->MatDotVec(A, x[s[0] + i], y[s[1] + i]);
}
/* src/gcge_ops.c:132-146 */
static void h_mv_axpby(double a, void **x, double b, void **y, int *s, int *e, ops_t *ops)
{
    for (int i = 0; i < e[0] - s[0]; ++i) ops->VecAxpby(a, x[s[0] + i], b, y[s[1] + i]);
}
/* src/gcge_ops.c:163-193: first column by a*x + 0*y, the rest accumulated with b = 1 */
static void h_mv_lincomb(void **x, void **y, int *s, int *e, double *a, int lda, void *dmat, int lddmat, ops_t *ops)
{
    (void)dmat; (void)lddmat;
    for (int jy = s[1]; jy < e[1]; ++jy) {
        const double *col = a + (size_t)(jy - s[1]) * lda;
        ops->VecAxpby(col[0], x[s[0]], 0.0, y[jy]);
        for (int ix = s[0] + 1; ix < e[0]; ++ix)
            ops->VecAxpby(col[ix - s[0]], x[ix], 1.0, y[jy]);
    }
}
/* src/gcge_ops.c:198-261 (MPI reduction omitted: one process) */
static void h_mv_inner(void **V, void **W, double *a, char *is_sym, int *s, int *e, int lda, ops_t *ops)
{
    if (strcmp(is_sym, "sym") == 0) {
        int len = e[1] - s[1];
        double *p = a;
        for (int iw = 0; iw < len; ++iw) {
            for (int iv = 0; iv <= iw; ++iv, ++p)
                ops->VecInnerProd(V[iv + s[0]], W[iw + s[1]], p);
            p += lda - (iw + 1);
        }
        for (int iw = 0; iw < len; ++iw)
            for (int iv = iw + 1; iv < len; ++iv)
                a[(size_t)iw * lda + iv] = a[(size_t)iv * lda + iw];
    } else {
        int skip = lda - (e[0] - s[0]);
        double *p = a;
        for (int iw = s[1]; iw < e[1]; ++iw) {
            for (int iv = s[0]; iv < e[0]; ++iv, ++p)
                ops->VecInnerProd(V[iv], W[iw], p);
            p += skip;
        }
    }
}
/* src/gcge_ops.c:285-300: exchange column handles */
static void h_mv_swap(void **a, void **b, int *s, int *e, ops_t *ops)
{
    (void)ops;
    for (int i = 0; i < e[0] - s[0]; ++i) {
        void *t = a[s[0] + i];
        a[s[0] + i] = b[s[1] + i];
        b[s[1] + i] = t;
    }
}

static void mv_matdot(void *A, mv_t *x, mv_t *y, const int *s, const int *e)
{
    int ss[2] = {s[0], s[1]}, ee[2] = {e[0], e[1]};
    T->MatDotMultiVec(A, x->c, y->c, ss, ee, T);
}
static void mv_axpby(double a, mv_t *x, double b, mv_t *y, const int *s, const int *e)
{
    int ss[2] = {s[0], s[1]}, ee[2] = {e[0], e[1]};
    T->MultiVecAxpby(a, x->c, b, y->c, ss, ee, T);
}
static void mv_lincomb(mv_t *x, mv_t *y, const int *s, const int *e, const double *a, int lda)
{
    int ss[2] = {s[0], s[1]}, ee[2] = {e[0], e[1]};
    T->MultiVecLinearComb(x->c, y->c, ss, ee, (double *)a, lda, NULL, 0, T);
}
static void mv_inner(mv_t *V, mv_t *W, double *a, int sym, const int *s, const int *e, int lda)
{
    int ss[2] = {s[0], s[1]}, ee[2] = {e[0], e[1]};
    char sy[] = "sym", ns[] = "nonsym";
    T->MultiVecInnerProd(V->c, W->c, a, sym ? sy : ns, ss, ee, lda, T);
}
static void mv_swap(mv_t *a, mv_t *b, const int *s, const int *e)
{
    int ss[2] = {s[0], s[1]}, ee[2] = {e[0], e[1]};
    T->MultiVecSwap(a->c, b->c, ss, ee, T);
}

/* dsyevx("V", "I", "U") of the projected problems, ops->DenseMatEigenSolver
 * (default src/gcge_ops.c:302-316) */
static void h_dsyevx(char *jobz, char *range, char *uplo, int *nrows, double *a, int *lda, double *vl, double *vu,
                     int *il, int *iu, double *abstol, int *nev, double *eval, double *evec, int *lde, int *isuppz,
                     double *work, int *lwork, int *iwork, int *liwork, int *ifail, int *info)
{
    (void)isuppz; (void)liwork;
    scipy_dsyevx_(jobz, range, uplo, nrows, a, lda, vl, vu, il, iu, abstol, nev, eval, evec, lde, work, lwork, iwork,
                  ifail, info);
}
static void dsyevx(char *jobz, char *range, char *uplo, int *nrows, double *a, int *lda, double *vl, double *vu,
                   int *il, int *iu, double *abstol, int *nev, double *eval, double *evec, int *lde, double *work,
                   int *lwork, int *iwork, int *ifail, int *info)
{
    int liwork = 0;
    T->DenseMatEigenSolver(jobz, range, uplo, nrows, a, lda, vl, vu, il, iu, abstol, nev, eval, evec, lde, NULL, work,
                           lwork, iwork, &liwork, ifail, info);
}

static void h_dirichlet(void **vecs, int nev, void *Av, void *Bv);

/* CSR_VecSetRandomValue, app/csr/gcge_app_csr.c:283-293: libc rand() / (RAND_MAX + 1) */
static void h_vec_random(void *v)
{
    hvec_t *x = (hvec_t *)v;
    for (int i = 0; i < x->size; ++i) x->e[i] = ((double)rand()) / ((double)RAND_MAX + 1);
}
/* GCGE_Default_MultiVecSetRandomValue, src/gcge_ops.c:102-112: column by column */
static void h_mv_random(void **mv, int start, int n_vec, ops_t *ops)
{
    for (int i = 0; i < n_vec; ++i) ops->VecSetRandomValue(mv[start + i]);
}
/* GCGE_Default_MultiVecCreateByMat / Destroy, src/gcge_ops.c:72-100: one vector
 * (its own storage) per handle, so that handles exchanged between multivectors
 * are each freed once, by whichever multivector holds them at the end */
static void h_mv_create_by_mat(void ***mv, int k, void *mat, ops_t *ops)
{
    (void)ops;
    const int n = ((const csr_t *)mat)->n;
    void **h = (void **)malloc(sizeof(void *) * (k > 0 ? k : 1));
    for (int j = 0; j < k; ++j) {
        hvec_t *v = (hvec_t *)malloc(sizeof(hvec_t));
        v->size = n;
        v->e = (double *)calloc((size_t)n, sizeof(double));
        h[j] = v;
    }
    *mv = h;
}
static void h_mv_destroy(void ***mv, int k, ops_t *ops)
{
    (void)ops;
    if (!mv || !*mv) return;
    for (int j = 0; j < k; ++j) {
        hvec_t *v = (hvec_t *)(*mv)[j];
        if (v) { free(v->e); free(v); }
    }
    free(*mv);
    *mv = NULL;
}

/* the reference's CSR table (GCGE_CSR_SetOps, app/csr/gcge_app_csr.c:70-84, plus the
 * defaults GCGE_OPS_Setup installs, src/gcge_ops.c:521-604) */
static ops_t H_OPS = {
    .MatDotVec = h_matvec, .VecAxpby = h_axpby, .VecInnerProd = h_dot, .VecLocalInnerProd = h_dot,
    .MatDotMultiVec = h_mv_matdot, .MultiVecAxpby = h_mv_axpby, .MultiVecLinearComb = h_mv_lincomb,
    .MultiVecInnerProd = h_mv_inner, .MultiVecSwap = h_mv_swap, .DenseMatEigenSolver = h_dsyevx,
    .SetDirichletBoundary = h_dirichlet, .VecSetRandomValue = h_vec_random, .MultiVecSetRandomValue = h_mv_random,
    .MultiVecCreateByMat = h_mv_create_by_mat, .MultiVecDestroy = h_mv_destroy,
};

static void use_host_table(void) { T = &H_OPS; g_host = 1; }

/* ------------------------------------------------------------------ state */
typedef struct {
    /* parameters (after GCGE_PARA_Setup, src/gcge_para.c:357-386) */
    int nev, block_size, ev_max_it, cg_max_it, max_reorth_time, dirichlet, print_level;
    double ev_tol, cg_rate, orth_zero_tol, reorth_tol, scbgs_reorth_tol, criterion_tol;
    double multi_tol_for_lock, conv_omega_norm;
    int opt_rr_eig_partly;
    char w_orth_type[8];
    char conv_type[4];
    /* para outputs */
    int num_unlock, num_iter;
    double max_res, min_res, sum_res;
    double *res;
    /* workspace (src/gcge_workspace.c:61-119) */
    int max_dim_x, dim_x, dim_xp, dim_xpw, last_dim_xpw, last_dim_x, unconv_bs, soft_locked;
    mv_t V, V_tmp, CG_p, evec;
    int *unlock;
    double *eval, *sub_dtmp, *sub_evec, *sub_mat;
    int *sub_itmp;
    void *A, *B;
} gcge_t;

/* ------------------------------------------------------- block CG (a8) */
/* GCGE_BCG, src/gcge_cg.c:137-302. CG_R = RHS, CG_P = p-block, CG_W = w-block,
 * CG_X = X[:, xs : xs+len]. The active list is rebuilt each iteration by writing
 * unlock[idx] = idx at position idx (src/gcge_cg.c:713-720), so the update loops,
 * which walk unlock[0 .. num_unlock), always touch the first num_unlock columns. */
static void bcg(void *A, mv_t *R, mv_t *X, int xs, int len, mv_t *P, mv_t *Wk,
                double *dtmp, int *itmp, int cg_max_it, double rate)
{
    double *rho1 = dtmp, *rho2 = rho1 + len, *err = rho2 + len, *lerr = err + len, *ptw = lerr + len;
    int *unlock = itmp, num_unlock = 0;
    for (int idx = 0; idx < len; ++idx) {
        csr_mv(A, X->c[xs + idx], Wk->c[idx]);
        vaxpby(-1.0, Wk->c[idx], 1.0, R->c[idx]);
        rho2[idx] = vdot(R->c[idx], R->c[idx]);
        unlock[idx] = idx;
        num_unlock++;
    }
    for (int idx = 0; idx < len; ++idx) err[idx] = sqrt(rho2[idx]);
    int niter = 1;
    while (num_unlock > 0 && niter < cg_max_it) {
        if (niter == 1) {
            for (int id = 0; id < num_unlock; ++id) {
                int idx = unlock[id];
                vaxpby(1.0, R->c[idx], 0.0, P->c[idx]);
            }
        } else {
            for (int id = 0; id < num_unlock; ++id) {
                int idx = unlock[id];
                double beta = rho2[idx] / rho1[idx];
                vaxpby(1.0, R->c[idx], beta, P->c[idx]);
            }
        }
        for (int id = 0; id < num_unlock; ++id) {
            int idx = unlock[id];
            csr_mv(A, P->c[idx], Wk->c[idx]);
            ptw[idx] = vdot(P->c[idx], Wk->c[idx]);
        }
        for (int id = 0; id < num_unlock; ++id) {
            int idx = unlock[id];
            double alpha = rho2[idx] / ptw[idx];
            vaxpby(alpha, P->c[idx], 1.0, X->c[xs + idx]);
            vaxpby(-alpha, Wk->c[idx], 1.0, R->c[idx]);
            rho1[idx] = rho2[idx];
            rho2[idx] = vdot(R->c[idx], R->c[idx]);
        }
        for (int idx = 0; idx < len; ++idx) lerr[idx] = sqrt(fabs(rho2[idx]));
        num_unlock = 0;
        for (int idx = 0; idx < len; ++idx)
            if (lerr[idx] / err[idx] >= rate) { unlock[idx] = idx; num_unlock++; }
        niter++;
    }
}

/* ------------------------------------------------ orthogonalisation (a10/a11) */
/* GCGE_Orthonormalization, src/gcge_orthogonal.c:112-305: vector-by-vector
 * B-orthonormalisation with re-orthogonalisation; the column (MGS) form is used when
 * 0 < sum_res < criterion_tol, the block (CGS) form otherwise. Returns the new end. */
static int orth_plain(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    double *d = g->sub_dtmp;
    double vin = 0.0, vout = 0.0, ratio;
    void *t0 = g->V_tmp.c[0], *t1 = g->V_tmp.c[1];
    for (int cur = start; cur < end; ++cur) {
        int reorth = 0;
        if (g->sum_res > 0.0 && g->sum_res < g->criterion_tol) {
            void *vc = V->c[cur];
            if (!B) vout = sqrt(vdot(vc, vc));
            else { csr_mv(B, vc, t1); vout = sqrt(vdot(vc, t1)); }
            do {
                for (int j = 0; j < cur; ++j) {
                    double ipv;
                    if (!B) ipv = vdot(vc, V->c[j]);
                    else { csr_mv(B, vc, t1); ipv = vdot(V->c[j], t1); }
                    vaxpby(-ipv, V->c[j], 1.0, vc);
                }
                vin = vout;
                double nv;
                if (!B) nv = vdot(vc, vc);
                else { csr_mv(B, vc, t1); nv = vdot(vc, t1); }
                vout = sqrt(nv);
                ratio = vout / vin;
                /* the reference never advances its counter on this path
                 * (src/gcge_orthogonal.c:207); the norm test ends the loop */
            } while (ratio < g->reorth_tol && reorth < g->max_reorth_time && vout > g->orth_zero_tol);
        } else {
            do {
                if (!B) vaxpby(1.0, V->c[cur], 0.0, t0);
                else csr_mv(B, V->c[cur], t0);
                int s[2] = {0, 0}, e[2] = {cur + 1, 1};
                mv_inner(V, &g->V_tmp, d, 0, s, e, cur + 1);
                if (cur != 0) {
                    int s2[2] = {0, 0}, e2[2] = {cur, 1};
                    mv_lincomb(V, &g->V_tmp, s2, e2, d, cur);
                    vaxpby(-1.0, t0, 1.0, V->c[cur]);
                }
                vin = sqrt(d[cur]);
                d[cur] = d[cur] - arr_dot(d, d, cur);
                vout = sqrt(d[cur]);
                ratio = vout / vin;
                reorth++;
            } while (ratio < g->reorth_tol && reorth < g->max_reorth_time && vout > g->orth_zero_tol);
        }
        if (vout > g->orth_zero_tol) {
            vaxpby(0.0, V->c[cur], 1.0 / vout, V->c[cur]);
        } else {
            int s[2] = {cur, end - 1}, e[2] = {cur + 1, end};
            mv_swap(V, V, s, e);
            end--;
            cur--;
        }
    }
    return end;
}

/* GCGE_BOrthonormalization, src/gcge_orthogonal.c:352-528 (w_orth_type "bgs"):
 * B V[:, 0:nev] into evec and B V[:, nev:dim_xp] into V_tmp once; then twice:
 * W[:, start:end) projected against each of X and P in turn (classical per
 * vector, V^T evec / V^T V_tmp), and W itself by modified Gram-Schmidt with its
 * B-norm; a column of norm <= orth_zero_tol is swapped to the end and dropped. */
static int bgs_orth(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    const int nev = g->nev, dim_xp = g->dim_xp;
    double *d = g->sub_dtmp;
    for (int j = 0; j < nev; ++j) {
        if (!B) vaxpby(1.0, V->c[j], 0.0, g->evec.c[j]);
        else csr_mv(B, V->c[j], g->evec.c[j]);
    }
    for (int j = nev; j < dim_xp; ++j) {
        if (!B) vaxpby(1.0, V->c[j], 0.0, g->V_tmp.c[j - nev]);
        else csr_mv(B, V->c[j], g->V_tmp.c[j - nev]);
    }
    for (int i = 0; i < 2; ++i) {
        int wl = end - start;
        for (int cur = 0; cur < nev; ++cur) {
            int s[2] = {start, cur}, e[2] = {end, cur + 1};
            mv_inner(V, &g->evec, d, 0, s, e, wl);
            for (int j = start; j < end; ++j) vaxpby(-d[j - start], V->c[cur], 1.0, V->c[j]);
        }
        for (int cur = nev; cur < dim_xp; ++cur) {
            int s[2] = {start, cur - nev}, e[2] = {end, cur + 1 - nev};
            mv_inner(V, &g->V_tmp, d, 0, s, e, wl);
            for (int j = start; j < end; ++j) vaxpby(-d[j - start], V->c[cur], 1.0, V->c[j]);
        }
        for (int cur = start; cur < end; cur++) {
            if (!B) vaxpby(1.0, V->c[cur], 0.0, g->CG_p.c[0]);
            else csr_mv(B, V->c[cur], g->CG_p.c[0]);
            int s[2] = {cur, 0}, e[2] = {end, 1};
            wl = end - cur;
            mv_inner(V, &g->CG_p, d, 0, s, e, wl);
            const double nv = sqrt(d[0]);
            if (nv > g->orth_zero_tol) {
                vaxpby(0.0, V->c[cur], 1.0 / nv, V->c[cur]);
                for (int j = cur + 1; j < end; ++j) vaxpby(-d[j - cur] / nv, V->c[cur], 1.0, V->c[j]);
            } else {
                int s2[2] = {cur, end - 1}, e2[2] = {cur + 1, end};
                mv_swap(V, V, s2, e2);
                end--;
                cur--;
            }
        }
    }
    return end;
}

/* GCGE_CBOrthonormalization, src/gcge_orthogonal.c:755-964 (w_orth_type "cbgs"):
 * two block passes W -= V (V^T B W) against V[:, 0:start), then once: the Gram
 * W^T B W, and if any entry exceeds orth_zero_tol its eigenpairs by dsyevx,
 * eigenvectors of eigenvalues >= orth_zero_tol scaled by theta^-1/2 (everything up
 * to the last smaller one dropped), W <- W Q (the linear combination's stride and
 * offset use the reduced count, as the reference does), swapped into V. */
static int cbgs_orth(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    const int w0 = end - start;
    double *d = g->sub_dtmp, *tmp_evec = g->sub_evec, *tmp_eval = tmp_evec + (size_t)w0 * w0;
    double *dwork = d + (size_t)w0 * w0;
    int *iwork = g->sub_itmp, *ifail = g->sub_itmp + 5 * w0;
    int wl = w0;
    for (int i = 0; i < 2; ++i) {
        wl = end - start;
        int s[2] = {start, 0}, e[2] = {end, wl};
        if (!B) mv_axpby(1.0, V, 0.0, &g->V_tmp, s, e);
        else mv_matdot(B, V, &g->V_tmp, s, e);
        int s1[2] = {0, 0}, e1[2] = {start, wl};
        mv_inner(V, &g->V_tmp, d, 0, s1, e1, start);
        mv_lincomb(V, &g->V_tmp, s1, e1, d, start);
        int s2[2] = {0, start}, e2[2] = {wl, end};
        mv_axpby(-1.0, &g->V_tmp, 1.0, V, s2, e2);
    }
    for (int j = 0; j < wl; ++j) {
        if (!B) vaxpby(1.0, V->c[j + start], 0.0, g->V_tmp.c[j]);
        else csr_mv(B, V->c[j + start], g->V_tmp.c[j]);
    }
    {
        int s[2] = {start, 0}, e[2] = {end, wl};
        mv_inner(V, &g->V_tmp, d, 0, s, e, wl);
    }
    int nonzero = 0;
    for (int j = 0; j < wl * wl; ++j)
        if (d[j] > g->orth_zero_tol) {
            nonzero = 1;
            break;
        }
    if (!nonzero) return start;
    double vl = 0.0, vu = 0.0, abstol = 0.0;
    int il = 1, iu = wl, m = iu - il + 1, lwork = 8 * w0, info = 0, nn = wl;
    char V_ = 'V', I_ = 'I', U_ = 'U';
    dsyevx(&V_, &I_, &U_, &nn, d, &nn, &vl, &vu, &il, &iu, &abstol, &m, tmp_eval, tmp_evec, &nn, dwork, &lwork,
                  iwork, ifail, &info);
    int nz = 0;
    for (int j = 0; j < wl; ++j) {
        if (tmp_eval[j] < g->orth_zero_tol) nz = j + 1;
        else arr_scal(1.0 / sqrt(tmp_eval[j]), tmp_evec + (size_t)j * wl, wl);
    }
    wl -= nz;
    {
        int s[2] = {start, 0}, e[2] = {end, wl};
        mv_lincomb(V, &g->V_tmp, s, e, tmp_evec + (size_t)nz * wl, wl);
    }
    end = start + wl;
    {
        int s[2] = {start, 0}, e[2] = {end, wl};
        mv_swap(V, &g->V_tmp, s, e);
    }
    return end;
}

/* GCGE_SCBOrth_Minus, src/gcge_orthogonal.c:1116-1195: W[:, start:end) -= the
 * projection onto V[:, dim_xp:start), repeated while the summed squares of the
 * first (start - dim_xp) * w entries of the Gram buffer exceed scbgs_reorth_tol
 * (the Gram is stored with leading dimension start, as the reference does) */
static void scb_minus(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    const int wl = end - start, dim_xp = g->dim_xp, length = (start - dim_xp) * wl;
    double *d = g->sub_dtmp, vi = 1.0;
    int iter = 0;
    while (vi > g->scbgs_reorth_tol) {
        iter++;
        int s[2] = {start, 0}, e[2] = {end, wl};
        if (!B) mv_axpby(1.0, V, 0.0, &g->V_tmp, s, e);
        else mv_matdot(B, V, &g->V_tmp, s, e);
        int s1[2] = {dim_xp, 0}, e1[2] = {start, wl};
        mv_inner(V, &g->V_tmp, d, 0, s1, e1, start);
        vi = 0.0;
        for (int i = 0; i < length; ++i) vi += d[i] * d[i];
        vi = sqrt(vi);
        mv_lincomb(V, &g->V_tmp, s1, e1, d, start);
        int s2[2] = {0, start}, e2[2] = {wl, end};
        mv_axpby(-1.0, &g->V_tmp, 1.0, V, s2, e2);
        if (iter >= g->max_reorth_time) break;
    }
}

/* GCGE_SCBOrth_Self, src/gcge_orthogonal.c:1196-1281: modified Gram-Schmidt in the
 * B inner product within W[:, start:end), scbgs_wself_max_reorth_time (1) times */
static int scb_self(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    double *d = g->sub_dtmp;
    for (int it = 0; it < 1; ++it) {
        for (int cur = start; cur < end; cur++) {
            if (!B) vaxpby(1.0, V->c[cur], 0.0, g->CG_p.c[0]);
            else csr_mv(B, V->c[cur], g->CG_p.c[0]);
            int s[2] = {cur, 0}, e[2] = {end, 1};
            mv_inner(V, &g->CG_p, d, 0, s, e, end - cur);
            const double nv = sqrt(d[0]);
            if (nv > g->orth_zero_tol) {
                vaxpby(0.0, V->c[cur], 1.0 / nv, V->c[cur]);
                for (int j = cur + 1; j < end; ++j) vaxpby(-d[j - cur] / nv, V->c[cur], 1.0, V->c[j]);
            } else {
                int s2[2] = {cur, end - 1}, e2[2] = {cur + 1, end};
                mv_swap(V, V, s2, e2);
                end--;
                cur--;
            }
        }
    }
    return end;
}

/* GCGE_SCBOrthonormalization, src/gcge_orthogonal.c:967-1115 (w_orth_type
 * "scbgs"): block projections of W against V[:, 0:start) while their norm exceeds
 * scbgs_reorth_tol (at most max_reorth_time), then W in blocks of
 * w_orth_block_size = max(block_size / 5, 1) (src/gcge_para.c:373-376): each block
 * projected against the W columns before it and orthonormalised by itself; columns
 * a block drops are swapped behind the remaining ones */
static int scbgs_orth(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    const int w0 = end - start, length = start * w0;
    double *d = g->sub_dtmp, vi = 1.0;
    int iter = 0;
    while (vi > g->scbgs_reorth_tol) {
        iter++;
        int s[2] = {start, 0}, e[2] = {end, w0};
        if (!B) mv_axpby(1.0, V, 0.0, &g->V_tmp, s, e);
        else mv_matdot(B, V, &g->V_tmp, s, e);
        int s1[2] = {0, 0}, e1[2] = {start, w0};
        mv_inner(V, &g->V_tmp, d, 0, s1, e1, start);
        vi = 0.0;
        for (int i = 0; i < length; ++i) vi += d[i] * d[i];
        vi = sqrt(vi);
        mv_lincomb(V, &g->V_tmp, s1, e1, d, start);
        int s2[2] = {0, start}, e2[2] = {w0, end};
        mv_axpby(-1.0, &g->V_tmp, 1.0, V, s2, e2);
        if (iter >= g->max_reorth_time) break;
    }
    const int bsz = g->block_size / 5 > 1 ? g->block_size / 5 : 1;
    const int step = (end - start) < bsz ? (end - start) : bsz;
    int ws = start, we = ws + step;
    if (we > end) we = end;
    we = scb_self(g, V, ws, we, B);
    while (we < end) {
        ws = we;
        we = ws + step;
        if (we > end) we = end;
        const int old_we = we;
        scb_minus(g, V, ws, we, B);
        we = scb_self(g, V, ws, we, B);
        if (we < old_we) {
            end -= old_we - we;
            int s2[2] = {we, end}, e2[2] = {old_we, end + old_we - we};
            mv_swap(V, V, s2, e2);
        }
    }
    return end;
}

/* GCGE_SubOrthonormalization, src/gcge_orthogonal.c:1880-1929:
 * V2 -= V1 (V1^T B V2), Gram left in sub_dtmp (len1 x len2, ld len1). */
static void sub_orth(gcge_t *g, mv_t *V, const int *s, const int *e, void *B)
{
    int len1 = e[0] - s[0], len2 = e[1] - s[1];
    int ms[2] = {s[1], 0}, me[2] = {e[1], len2};
    if (!B) mv_axpby(1.0, V, 0.0, &g->V_tmp, ms, me);
    else mv_matdot(B, V, &g->V_tmp, ms, me);
    int is[2] = {s[0], 0}, ie[2] = {e[0], len2};
    mv_inner(V, &g->V_tmp, g->sub_dtmp, 0, is, ie, len1);
    mv_lincomb(V, &g->V_tmp, is, ie, g->sub_dtmp, len1);
    int as[2] = {0, s[1]}, ae[2] = {len2, e[1]};
    mv_axpby(-1.0, &g->V_tmp, 1.0, V, as, ae);
}

/* GCGE_SubOrthonormalizationSelfBGS, src/gcge_orthogonal.c:2035-2115 */
static int self_bgs(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    double *d = g->sub_dtmp;
    void *t0 = g->V_tmp.c[0];
    for (int cur = start; cur < end; ++cur) {
        if (!B) vaxpby(1.0, V->c[cur], 0.0, t0);
        else csr_mv(B, V->c[cur], t0);
        int s[2] = {cur, 0}, e[2] = {end, 1};
        mv_inner(V, &g->V_tmp, d, 0, s, e, end - cur);
        double nrm = sqrt(d[0]);
        if (nrm > g->orth_zero_tol) {
            vaxpby(0.0, V->c[cur], 1.0 / nrm, V->c[cur]);
            for (int j = cur + 1; j < end; ++j)
                vaxpby(-d[j - cur] / nrm, V->c[cur], 1.0, V->c[j]);
        } else {
            int s2[2] = {cur, end - 1}, e2[2] = {cur + 1, end};
            mv_swap(V, V, s2, e2);
            end--;
            cur--;
        }
    }
    return end;
}

/* GCGE_MultiOrthonormalization, src/gcge_orthogonal.c:1945-2033: recursive
 * bisection; leaves (length <= max_direct_orth_length = 1) go to SelfBGS. */
static int multi_orth(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    int length = end - start;
    int l1 = length / 2, l2 = length - l1, mid = start + l1;
    if (length <= 1) return self_bgs(g, V, start, end, B);
    mid = multi_orth(g, V, start, mid, B);
    if (mid + l2 < end) {
        int new_end_2 = mid + l2, n_zero = end - new_end_2;
        int s[2] = {mid, new_end_2}, e[2] = {mid + n_zero, end};
        mv_swap(V, V, s, e);
        end = new_end_2;
    }
    if (mid - start > 0) {
        double value_inner = 1.0;
        int iter = 0;
        while (value_inner > g->scbgs_reorth_tol) {
            iter++;
            int s[2] = {start, mid}, e[2] = {mid, end};
            sub_orth(g, V, s, e, B);
            value_inner = 0.0;
            for (int i = 0; i < l1 * l2; ++i) value_inner += g->sub_dtmp[i] * g->sub_dtmp[i];
            value_inner = sqrt(value_inner);
            if (iter >= g->max_reorth_time) break;
        }
    }
    return multi_orth(g, V, mid, end, B);
}

/* GCGE_StableMultiOrthonormalization, src/gcge_orthogonal.c:1833-1877 */
static int stable_multi_orth(gcge_t *g, mv_t *V, int start, int end, void *B)
{
    double value_inner = 1.0;
    int iter = 0;
    while (value_inner > g->scbgs_reorth_tol) {
        iter++;
        int s[2] = {0, start}, e[2] = {start, end};
        sub_orth(g, V, s, e, B);
        value_inner = 0.0;
        for (int i = 0; i < start * (end - start); ++i) value_inner += g->sub_dtmp[i] * g->sub_dtmp[i];
        value_inner = sqrt(value_inner);
        if (iter >= g->max_reorth_time) break;
    }
    return multi_orth(g, V, start, end, B);
}

/* GCGE_MultiOrthonormalizationInSubspace, src/gcge_orthogonal.c:2130-2204 (B = I) */
static int multi_orth_sub(gcge_t *g, double *V, int ldV, int nrows, int start, int end)
{
    int length = end - start;
    int l1 = length / 2, l2 = length - l1, mid = start + l1;
    if (length == 1) {
        double nv = arr_nrm2(V + (size_t)start * ldV, nrows);
        if (nv > g->orth_zero_tol) arr_scal(1.0 / nv, V + (size_t)start * ldV, nrows);
        else end = start;
        return end;
    }
    mid = multi_orth_sub(g, V, ldV, nrows, start, mid);
    if (mid + l2 < end) {
        int new_end_2 = mid + l2, n_zero = end - new_end_2;
        l1 -= n_zero;
        memcpy(V + (size_t)mid * ldV, V + (size_t)new_end_2 * ldV, (size_t)n_zero * ldV * sizeof(double));
        end = new_end_2;
    }
    if (l1 > 0) {
        for (int r = 0; r < g->max_reorth_time; ++r) {
            dgemm('T', 'N', l1, l2, nrows, 1.0, V + (size_t)start * ldV, ldV,
                  V + (size_t)mid * ldV, ldV, 0.0, g->sub_dtmp, l1);
            dgemm('N', 'N', ldV, l2, l1, -1.0, V + (size_t)start * ldV, ldV,
                  g->sub_dtmp, l1, 1.0, V + (size_t)mid * ldV, ldV);
        }
    }
    return multi_orth_sub(g, V, ldV, nrows, mid, end);
}

/* GCGE_StableMultiOrthonormalizationInSubspace, src/gcge_orthogonal.c:2215-2247 */
static int stable_multi_orth_sub(gcge_t *g, double *V, int ldV, int nrows, int start, int end)
{
    if (start != 0) {
        for (int r = 0; r < g->max_reorth_time; ++r) {
            int len = end - start;
            dgemm('T', 'N', start, len, nrows, 1.0, V, ldV, V + (size_t)start * ldV, ldV,
                  0.0, g->sub_dtmp, start);
            dgemm('N', 'N', ldV, len, start, -1.0, V, ldV, g->sub_dtmp, start, 1.0,
                  V + (size_t)start * ldV, ldV);
        }
    }
    return multi_orth_sub(g, V, ldV, nrows, start, end);
}

/* ----------------------------------------------------- Rayleigh-Ritz (a16/a17) */
/* GCGE_ComputeSubspaceMatrixVTAW, src/gcge_rayleighritz.c:35-81 */
static void rr_vtaw(gcge_t *g, void *A, int start_W, int end_V, double *sub)
{
    int w_len = end_V - start_W, xp_len = end_V - w_len;
    int s[2] = {start_W, 0}, e[2] = {end_V, w_len};
    mv_matdot(A, &g->V, &g->evec, s, e);
    int s2[2] = {0, 0}, e2[2] = {xp_len, w_len};
    mv_inner(&g->V, &g->evec, sub, 0, s2, e2, end_V);
    mv_inner(&g->V, &g->evec, sub + xp_len, 1, s, e, end_V);
}

/* GCGE_ComputeSubspaceMatrix, src/gcge_rayleighritz.c:113-200 (structured form) */
static void rr_matrix(gcge_t *g, void *A)
{
    int dim_xp = g->dim_xp, ldm = g->dim_xpw;
    if (dim_xp != 0) {
        int lde = g->last_dim_xpw, dim_x = g->dim_x, dim_p = dim_xp - dim_x;
        double one = 1.0, zero = 0.0;
        double *pp = g->sub_evec + (size_t)dim_x * lde;
        char L = 'L', U = 'U';
        scipy_dsymm_(&L, &U, &lde, &dim_p, &one, g->sub_mat, &lde, pp, &lde, &zero, g->sub_dtmp, &lde);
        memset(g->sub_mat, 0, (size_t)ldm * ldm * sizeof(double));
        dgemm('T', 'N', dim_p, dim_p, lde, 1.0, pp, lde, g->sub_dtmp, lde, 0.0,
              g->sub_mat + (size_t)dim_x * ldm + dim_x, ldm);
        for (int i = 0; i < dim_x; ++i) g->sub_mat[(size_t)i * ldm + i] = g->eval[i];
    }
    rr_vtaw(g, A, dim_xp, ldm, g->sub_mat + (size_t)dim_xp * ldm);
}

/* GCGE_ComputeSubspaceEigenpairs, src/gcge_rayleighritz.c:364-590, single-process
 * path: with opt_rr_eig_partly the lock count is the first unconverged index,
 * lowered by every earlier eigenvalue within multi_tol_for_lock of it
 * (:378-394); the W columns' rows above it are zeroed in the projected matrix
 * (:408-409), and dsyevx("V","I","U") solves the trailing block for the pairs
 * lock+1 .. min(max_dim_x, ldm), writing eval and the coefficient columns from
 * the lock count on (:522-546). Without it the lock count is 0. */
static int rr_eig(gcge_t *g)
{
    int ldm = g->dim_xpw;
    double *tmp = g->sub_dtmp, *work = tmp + (size_t)ldm * ldm;
    double vl = 0.0, vu = 0.0, abstol = 0.0;
    int start = g->opt_rr_eig_partly ? g->unlock[0] : 0;
    int il = start;
    for (int i = start - 1; i > -1; --i)
        if (fabs(g->eval[i] - g->eval[start]) / g->eval[start] < g->multi_tol_for_lock) il -= 1;
    start = il;
    il += 1;
    g->soft_locked = start;
    int iu = g->max_dim_x < ldm ? g->max_dim_x : ldm, m = iu - il + 1;
    int lwork = 8 * ldm, info = 0, nrows = ldm, ncols = ldm;
    int *iwork = g->sub_itmp, *ifail = g->sub_itmp + 5 * ldm;
    for (int i = 0; i < g->dim_xpw - g->dim_xp; ++i)
        memset(g->sub_mat + (size_t)(g->dim_xp + i) * ldm, 0, (size_t)start * sizeof(double));
    memcpy(tmp, g->sub_mat, (size_t)ldm * ldm * sizeof(double));
    nrows -= start;
    il -= start;
    iu -= start;
    char V = 'V', I = 'I', U = 'U';
    dsyevx(&V, &I, &U, &nrows, tmp + (size_t)start * ncols + start, &ncols, &vl, &vu, &il, &iu, &abstol, &m,
                  g->eval + start, g->sub_evec + (size_t)start * ldm + start, &ldm, work, &lwork, iwork, ifail,
                  &info);
    return info;
}

/* -------------------------------------------------------- X, P, W (a9/a14/a15) */
/* GCGE_ComputeX, src/gcge_xpw.c:47-76 */
static void compute_x(gcge_t *g, int size_x, int size_v)
{
    int sx = g->soft_locked;
    int s[2] = {sx, sx}, e[2] = {size_v, size_x};
    mv_lincomb(&g->V, &g->evec, s, e, g->sub_evec + (size_t)sx * size_v + sx, size_v);
}

/* GCGE_ComputeW, src/gcge_xpw.c:118-217 (built-in block CG, no external solver) */
static void compute_w(gcge_t *g, void *A, void *B)
{
    int ws = g->dim_xp, wl = g->unconv_bs;
    for (int idx = 0; idx < wl; ++idx) {
        void *rhs = g->V_tmp.c[idx];
        int xi = g->unlock[idx];
        void *x = g->V.c[xi], *w = g->V.c[ws + idx];
        if (!B) vaxpby(1.0, x, 0.0, rhs);
        else csr_mv(B, x, rhs);
        double lam = g->eval[xi];
        if (fabs(lam) <= 1.0) {
            vaxpby(0.0, rhs, lam, rhs);
            vaxpby(1.0, x, 0.0, w);
        } else {
            vaxpby(1.0 / lam, x, 0.0, w);
        }
    }
    bcg(A, &g->V_tmp, &g->V, ws, wl, &g->CG_p, &g->evec, g->sub_dtmp, g->sub_itmp,
        g->cg_max_it, g->cg_rate);
}

/* GCGE_ComputeP, src/gcge_xpw.c:286-425 */
static void compute_p(gcge_t *g)
{
    double *coef = g->sub_evec;
    int ldc = g->dim_xpw, p_start = g->dim_x, p_ncols = g->unconv_bs, xx_nrows = g->last_dim_x;
    double *px = coef + (size_t)p_start * ldc, *pp = px + xx_nrows, *xp = coef + xx_nrows;
    memset(px, 0, (size_t)p_ncols * ldc * sizeof(double));
    for (int cp = 0; cp < p_ncols; ++cp)
        memcpy(pp + (size_t)cp * ldc, xp + (size_t)g->unlock[cp] * ldc,
               (size_t)(ldc - xx_nrows) * sizeof(double));
    int orth_start = g->soft_locked, orth_len = ldc - orth_start;
    p_start -= orth_start;
    int p_end = p_start + p_ncols;
    p_end = stable_multi_orth_sub(g, coef + (size_t)orth_start * ldc + orth_start, ldc, orth_len,
                                  p_start, p_end);
    p_end += orth_start;
    int p_end_tmp = p_end - g->nev;
    int s[2] = {orth_start, 0}, e[2] = {ldc, p_end_tmp};
    mv_lincomb(&g->V, &g->V_tmp, s, e, coef + (size_t)g->nev * ldc + orth_start, ldc);
    int s2[2] = {g->nev, 0}, e2[2] = {p_end, p_end_tmp};
    mv_swap(&g->V, &g->V_tmp, s2, e2);
    g->dim_xp = p_end;
}

/* ------------------------------------------------------ convergence (a18/a19) */
/* GCGE_CheckConvergence, src/gcge_eigsol.c:559-686, plus the "BR" criterion */
static void check_conv(gcge_t *g, void *A, void *B)
{
    int unconv = 0, max_conv_idx = 0, num_unlock = g->num_unlock;
    double max_res = 0.0, min_res = 0.0, sum_res = 0.0;
    void *t1 = g->V_tmp.c[0], *t2 = g->V_tmp.c[1];
    for (int j = 0; j < num_unlock; ++j) {
        int i = g->unlock[j];
        void *ev = g->evec.c[i];
        double lam = g->eval[i], bxn = 0.0;
        csr_mv(A, ev, t1);
        if (!B) { vaxpby(-lam, ev, 1.0, t1); }
        else { csr_mv(B, ev, t2); vaxpby(-lam, t2, 1.0, t1); }
        double rn = sqrt(vdot(t1, t1));
        double en = sqrt(vdot(ev, ev));
        double r;
        if (strcmp(g->conv_type, "R") == 0) r = rn / en / (1.0 > fabs(lam) ? 1.0 : fabs(lam));
        else if (strcmp(g->conv_type, "O") == 0) r = rn / en / (g->conv_omega_norm + fabs(lam));
        else if (strcmp(g->conv_type, "BR") == 0) {
            bxn = B ? sqrt(vdot(t2, t2)) : en;
            r = rn / (fabs(lam) * bxn);
        } else r = rn / en;
        g->res[i] = r;
        sum_res += r;
        if (j == 0) { max_res = r; min_res = r; }
        else { if (r > max_res) max_res = r; if (r < min_res) min_res = r; }
        if (r > g->ev_tol) {
            g->unlock[unconv++] = i;
            if (j > max_conv_idx + 8) {
                for (int k = j + 1; k < num_unlock; ++k) g->unlock[unconv++] = g->unlock[k];
                j = num_unlock + 1;
            }
        } else {
            max_conv_idx = j;
        }
    }
    g->num_unlock = unconv;
    g->unconv_bs = unconv < g->block_size ? unconv : g->block_size;
    g->max_res = max_res; g->min_res = min_res; g->sum_res = sum_res;
    g->num_iter += 1;
    if (g->print_level > 0)
        printf("num_unlock(%3d) = %3d; max_res(%3d) = %e; min_res(%3d) = %e;\n",
               g->num_iter, g->num_unlock, g->num_iter, max_res, g->num_iter, min_res);
}

/* GCGE_CheckEvalMultiplicity, src/gcge_eigsol.c:696-718 */
static int check_multiplicity(int nev, int end, const double *eval)
{
    int t = nev;
    for (int i = nev; i < end; ++i) {
        if (fabs(fabs(eval[t] / eval[nev]) - 1) < 0.2) t += 1;
        else break;
    }
    return t;
}

/* CSR_SetDirichletBoundary, app/csr/gcge_app_csr.c:130-183: rows where B has no
 * nonzero and A a single one are Dirichlet rows; the vectors are zeroed there */
static void h_dirichlet(void **vecs, int nev, void *Av, void *Bv)
{
    const csr_t *A = (const csr_t *)Av, *B = (const csr_t *)Bv;
    if (!A || !B) return;
    for (int i = 0; i < A->n; ++i) {
        int zero_b = 1;
        for (int j = B->rp[i]; j < B->rp[i + 1]; ++j)
            if (fabs(B->v[j]) > 1e-20) { zero_b = 0; break; }
        if (!zero_b) continue;
        int cnt = 0;
        for (int j = A->rp[i]; j < A->rp[i + 1]; ++j)
            if (fabs(A->v[j]) > 1e-20) cnt++;
        if (cnt == 1)
            for (int k = 0; k < nev; ++k) hcol(vecs[k])[i] = 0.0;
    }
}

/* ops->SetDirichletBoundary(evec, nev, A, B), src/gcge_eigsol.c:176-179 */
static void dirichlet_zero(gcge_t *g, void *A, void *B)
{
    if (!A || !B) return;
    T->SetDirichletBoundary(g->evec.c, g->nev, A, B);
}

/* ------------------------------------------------------------------ solve */
void gcge_oracle_default_params(gcge_oracle_params *p)
{
    memset(p, 0, sizeof(*p));
    p->nev = 1; p->block_size = 0; p->ev_max_it = 30; p->cg_max_it = 20; p->max_reorth_time = 3;
    p->ev_tol = 1e-8; p->cg_rate = 1e-2; p->orth_zero_tol = 1e-16; p->reorth_tol = 0.75;
    p->scbgs_reorth_tol = 1e-16; p->criterion_tol = 1e-6;
    strcpy(p->conv_type, "R");
    p->init_rng = 0; p->seed = 1;
}

/* ops->MultiVecSetRandomValue(evec, start, count), src/gcge_eigsol.c:131-134: on
 * the host table libc rand() after srand(seed) (CSR_VecSetRandomValue,
 * app/csr/gcge_app_csr.c:284-294) or the counter hash; a caller's table draws
 * from its own generator */
static void random_columns(gcge_t *g, const gcge_oracle_params *p, int from, int count)
{
    if (!g_host) {
        T->MultiVecSetRandomValue(g->evec.c, from, count, T);
        return;
    }
    int n = g->evec.n;
    for (int j = from; j < from + count; ++j) {
        double *c = hcol(g->evec.c[j]);
        if (p->init_rng == 0) {
            for (int i = 0; i < n; ++i) c[i] = ((double)rand()) / ((double)RAND_MAX + 1);
        } else {
            for (int i = 0; i < n; ++i)
                c[i] = gcge_oracle_hash_uniform(p->seed, (unsigned long long)j * n + i);
        }
    }
}

/* GCGE_Solve, src/gcge_eigsol.c:65-542, over the current table. evec is the
 * solver's eigenvector multivector (nev columns; the initial vectors when
 * given_init_evec = 1), eval_out[nev] the eigenvalues. */
static int solve_core(void *A, void *B, int n, const gcge_oracle_params *p, double *eval_out, mv_t *evec,
                      double *host_evec_out, gcge_oracle_stats *st)
{
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    gcge_t G, *g = &G;
    memset(g, 0, sizeof(G));
    g->A = A; g->B = B;
    /* GCGE_PARA_Setup, src/gcge_para.c:357-386 */
    int nev = p->nev;
    g->nev = nev;
    g->block_size = p->block_size ? p->block_size : nev;
    g->ev_max_it = p->ev_max_it; g->cg_max_it = p->cg_max_it; g->max_reorth_time = p->max_reorth_time;
    g->dirichlet = p->dirichlet_boundary; g->print_level = p->print_level;
    g->opt_rr_eig_partly = p->opt_rr_eig_partly;
    snprintf(g->w_orth_type, sizeof g->w_orth_type, "%.7s", p->w_orth_type[0] ? p->w_orth_type : "multi");
    g->multi_tol_for_lock = 1e-6;                 /* src/gcge_para.c:59 */
    g->ev_tol = p->ev_tol; g->cg_rate = p->cg_rate;
    g->orth_zero_tol = p->orth_zero_tol + DBL_EPSILON;
    g->reorth_tol = p->reorth_tol;
    g->scbgs_reorth_tol = p->scbgs_reorth_tol + DBL_EPSILON;
    g->criterion_tol = p->criterion_tol;
    snprintf(g->conv_type, sizeof g->conv_type, "%.3s", p->conv_type);
    g->num_unlock = nev;
    g->res = (double *)malloc(sizeof(double) * nev);
    for (int i = 0; i < nev; ++i) g->res[i] = 1.0;
    /* GCGE_WORKSPACE_Setup, src/gcge_workspace.c:61-119 */
    int mtmp = (nev * 1.25 < nev + 8) ? (int)(nev * 1.25) : (nev + 8);
    int max_dim_x = mtmp > nev + 3 ? mtmp : nev + 3;
    int bs = g->block_size;
    int V_size = max_dim_x + 2 * bs, Vt_size = max_dim_x - nev + bs, max_dim_xpw = V_size;
    mv_alloc(&g->V, A, n, V_size);
    mv_alloc(&g->V_tmp, A, n, Vt_size);
    mv_alloc(&g->CG_p, A, n, bs);
    g->evec = *evec;
    g->max_dim_x = max_dim_x; g->dim_x = nev; g->dim_xp = 0; g->dim_xpw = nev;
    g->unconv_bs = nev < bs ? nev : bs;
    g->eval = (double *)calloc(max_dim_xpw, sizeof(double));
    g->sub_dtmp = (double *)calloc((size_t)max_dim_xpw * max_dim_xpw + 40 * (size_t)max_dim_xpw, sizeof(double));
    g->sub_itmp = (int *)calloc(100 * (size_t)max_dim_xpw, sizeof(int));
    g->sub_evec = (double *)calloc((size_t)max_dim_xpw * max_dim_xpw, sizeof(double));
    g->sub_mat = (double *)calloc((size_t)max_dim_xpw * max_dim_xpw, sizeof(double));
    g->unlock = (int *)calloc(max_dim_x, sizeof(int));
    for (int i = 0; i < max_dim_x; ++i) g->unlock[i] = i;

    if (p->init_rng == 0) srand((unsigned)p->seed);
    int status = 0;

    /* initial X, src/gcge_eigsol.c:126-207 */
    if (p->given_init_evec == 0) {
        int num_init = 0;
        int guard = 0;
        do {
            random_columns(g, p, num_init, nev - num_init);
            if (strcmp(g->conv_type, "O") == 0 && num_init == 0) {
                double omega = 0.0, aomega = 0.0;
                for (int i = 0; i < nev; ++i) {
                    double nv = vdot(g->evec.c[i], g->evec.c[i]);
                    vaxpby(0.0, g->evec.c[i], 1.0 / sqrt(nv), g->evec.c[i]);
                }
                for (int i = 0; i < nev; ++i) omega += vdot(g->evec.c[i], g->evec.c[i]);
                int s[2] = {0, 0}, e[2] = {nev, nev};
                mv_matdot(A, &g->evec, &g->V, s, e);
                for (int i = 0; i < nev; ++i) aomega += vdot(g->V.c[i], g->V.c[i]);
                g->conv_omega_norm = sqrt(aomega / omega);
            }
            if (g->dirichlet) dirichlet_zero(g, A, B);
            g->dim_x = nev;
            g->dim_x = orth_plain(g, &g->evec, num_init, g->dim_x, B);
            num_init = g->dim_x;
            if (++guard > 100) { status = 2; break; }
        } while (num_init < nev);
    } else {
        g->dim_x = orth_plain(g, &g->evec, 0, nev, B);
    }
    {
        int s[2] = {0, 0}, e[2] = {nev, nev};
        mv_axpby(1.0, &g->evec, 0.0, &g->V, s, e);
    }
    g->dim_xpw = g->dim_x;
    g->last_dim_x = g->dim_x;
    g->dim_xp = 0;
    rr_matrix(g, A);
    if (rr_eig(g)) status = 3;
    compute_x(g, nev, g->dim_xpw);
    check_conv(g, A, B);
    {
        int s[2] = {g->soft_locked, g->soft_locked}, e[2] = {nev, nev};
        mv_swap(&g->V, &g->evec, s, e);
    }
    g->dim_xp = g->dim_x;
    compute_w(g, A, B);
    g->last_dim_xpw = g->dim_xpw;
    g->dim_xpw = g->dim_xp + g->unconv_bs;
    g->dim_xpw = orth_plain(g, &g->V, g->dim_x, g->dim_xpw, B);
    g->dim_xp = nev;
    rr_matrix(g, A);
    if (rr_eig(g)) status = 3;
    compute_x(g, nev, g->dim_xpw);
    check_conv(g, A, B);

    /* main loop, src/gcge_eigsol.c:396-528 */
    while (g->num_unlock > 0 && g->num_iter < g->ev_max_it) {
        compute_p(g);
        {
            int s[2] = {g->soft_locked, g->soft_locked}, e[2] = {nev, nev};
            mv_swap(&g->V, &g->evec, s, e);
        }
        compute_w(g, A, B);
        g->last_dim_xpw = g->dim_xpw;
        g->dim_xpw = g->dim_xp + g->unconv_bs;
        /* w_orth_type dispatch, src/gcge_eigsol.c:448-472 */
        if (strcmp(g->w_orth_type, "multi") == 0)
            g->dim_xpw = stable_multi_orth(g, &g->V, g->dim_xp, g->dim_xpw, B);
        else if (strcmp(g->w_orth_type, "bgs") == 0)
            g->dim_xpw = bgs_orth(g, &g->V, g->dim_xp, g->dim_xpw, B);
        else if (strcmp(g->w_orth_type, "cbgs") == 0)
            g->dim_xpw = cbgs_orth(g, &g->V, g->dim_xp, g->dim_xpw, B);
        else if (strcmp(g->w_orth_type, "scbgs") == 0)
            g->dim_xpw = scbgs_orth(g, &g->V, g->dim_xp, g->dim_xpw, B);
        else
            g->dim_xpw = orth_plain(g, &g->V, g->dim_xp, g->dim_xpw, B);
        rr_matrix(g, A);
        if (rr_eig(g)) status = 3;
        g->last_dim_x = g->dim_x;
        g->dim_x = check_multiplicity(nev, max_dim_x, g->eval);
        compute_x(g, nev, g->dim_xpw);
        check_conv(g, A, B);
    }

    /* the soft-locked Ritz vectors live in V: copied to evec at exit (src/gcge_eigsol.c:531-538) */
    if (g->soft_locked > 0) {
        int s[2] = {0, 0}, e[2] = {g->soft_locked, g->soft_locked};
        mv_axpby(1.0, &g->V, 0.0, &g->evec, s, e);
    }
    memcpy(eval_out, g->eval, sizeof(double) * nev);
    /* host table: column j of the result is the handle in position j (swaps
     * exchange handles, so it may live in the workspace freed below) */
    if (g_host && host_evec_out)
        for (int j = 0; j < nev; ++j) memcpy(host_evec_out + (size_t)j * n, hcol(g->evec.c[j]), sizeof(double) * n);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    if (st) {
        st->num_iter = g->num_iter; st->num_unlock = g->num_unlock;
        st->max_res = g->max_res; st->min_res = g->min_res; st->sum_res = g->sum_res;
        st->wall_s = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
        st->status = status;
    }
    mv_free(&g->V); mv_free(&g->V_tmp); mv_free(&g->CG_p);
    free(g->eval); free(g->sub_dtmp); free(g->sub_itmp); free(g->sub_evec); free(g->sub_mat);
    free(g->unlock); free(g->res);
    return status;
}

int gcge_oracle_solve(int n, const int *A_rp, const int *A_ci, const double *A_v,
                      const int *B_rp, const int *B_ci, const double *B_v,
                      const gcge_oracle_params *p, double *eval_out, double *evec_out,
                      gcge_oracle_stats *st)
{
    use_host_table();
    csr_t Am = {n, A_rp, A_ci, A_v}, Bm = {n, B_rp, B_ci, B_v};
    mv_t ev;
    h_mv_make(&ev, n, p->nev, NULL);
    if (p->given_init_evec)
        for (int j = 0; j < p->nev; ++j) memcpy(hcol(ev.c[j]), evec_out + (size_t)j * n, sizeof(double) * n);
    int status = solve_core(&Am, B_rp ? &Bm : NULL, n, p, eval_out, &ev, evec_out, st);
    h_mv_free(&ev);
    return status;
}

int gcge_oracle_solve_table(void *ops_table, void *A, void *B, int n, const gcge_oracle_params *p, double *eval_out,
                            void **evec, gcge_oracle_stats *st)
{
    ops_t *ops = (ops_t *)ops_table;
    if (!ops || !A || !evec || n <= 0 || p->nev <= 0) return 1;
    /* the members GCGE_OPS_Setup requires (src/gcge_ops.c:473-520) and the block
     * members this restatement calls */
    if (!ops->MatDotVec || !ops->VecAxpby || !ops->VecInnerProd || !ops->MatDotMultiVec || !ops->MultiVecAxpby ||
        !ops->MultiVecLinearComb || !ops->MultiVecInnerProd || !ops->MultiVecSwap || !ops->MultiVecCreateByMat ||
        !ops->MultiVecDestroy || !ops->MultiVecSetRandomValue || !ops->DenseMatEigenSolver ||
        (p->dirichlet_boundary && !ops->SetDirichletBoundary))
        return 1;
    T = ops;
    g_host = 0;
    mv_t ev = {n, p->nev, evec, NULL, NULL};
    int status = solve_core(A, B, n, p, eval_out, &ev, NULL, st);
    use_host_table();
    return status;
}

/* --------------------------------------------------------- single-op entries */
void gcge_oracle_csr_matvec(int n, const int *rp, const int *ci, const double *v,
                            const double *x, double *y)
{
    use_host_table();
    csr_t A = {n, rp, ci, v};
    hvec_t xv = {n, (double *)x}, yv = {n, y};
    csr_mv(&A, &xv, &yv);
}

void gcge_oracle_csr_matmultivec(int n, int k, const int *rp, const int *ci, const double *v,
                                 const double *X, double *Y)
{
    use_host_table();
    csr_t A = {n, rp, ci, v};
    mv_t x, y;
    h_mv_make(&x, n, k, (double *)X);
    h_mv_make(&y, n, k, Y);
    int s[2] = {0, 0}, e[2] = {k, k};
    mv_matdot(&A, &x, &y, s, e);
    h_mv_free(&x); h_mv_free(&y);
}

void gcge_oracle_vec_axpby(int n, double a, const double *x, double b, double *y)
{
    use_host_table();
    hvec_t xv = {n, (double *)x}, yv = {n, y};
    vaxpby(a, &xv, b, &yv);
}

void gcge_oracle_multivec_lincomb(int n, int nx, int ny, const double *X, double *Y,
                                  const double *coef, int lda)
{
    use_host_table();
    mv_t x, y;
    h_mv_make(&x, n, nx, (double *)X);
    h_mv_make(&y, n, ny, Y);
    int s[2] = {0, 0}, e[2] = {nx, ny};
    mv_lincomb(&x, &y, s, e, coef, lda);
    h_mv_free(&x); h_mv_free(&y);
}

void gcge_oracle_multivec_innerprod(int n, int nv, int nw, const double *V, const double *W,
                                    double *a, int lda, int sym)
{
    use_host_table();
    mv_t v, w;
    h_mv_make(&v, n, nv, (double *)V);
    h_mv_make(&w, n, nw, (double *)W);
    int s[2] = {0, 0}, e[2] = {nv, nw};
    mv_inner(&v, &w, a, sym, s, e, lda);
    h_mv_free(&v); h_mv_free(&w);
}

void gcge_oracle_bcg(int n, int k, const int *rp, const int *ci, const double *v,
                     double *RHS, double *W, int cg_max_it, double cg_rate)
{
    use_host_table();
    csr_t A = {n, rp, ci, v};
    mv_t R, X, P, Wk;
    h_mv_make(&R, n, k, RHS);
    h_mv_make(&X, n, k, W);
    h_mv_make(&P, n, k, NULL);
    h_mv_make(&Wk, n, k, NULL);
    double *dtmp = (double *)calloc(6 * (size_t)(k + 1), sizeof(double));
    int *itmp = (int *)calloc(k + 1, sizeof(int));
    bcg(&A, &R, &X, 0, k, &P, &Wk, dtmp, itmp, cg_max_it, cg_rate);
    free(dtmp); free(itmp);
    h_mv_free(&P); h_mv_free(&Wk); h_mv_free(&R); h_mv_free(&X);
}

int gcge_oracle_stable_multi_orth(int n, int ncols, double *Vd, int start, int end,
                                  const int *B_rp, const int *B_ci, const double *B_v,
                                  int max_reorth_time, double orth_zero_tol, double scbgs_reorth_tol)
{
    use_host_table();
    csr_t Bm = {n, B_rp, B_ci, B_v};
    gcge_t G;
    memset(&G, 0, sizeof(G));
    G.max_reorth_time = max_reorth_time;
    G.orth_zero_tol = orth_zero_tol + DBL_EPSILON;
    G.scbgs_reorth_tol = scbgs_reorth_tol + DBL_EPSILON;
    mv_t V;
    h_mv_make(&V, n, ncols, Vd);
    int width = end - start > 1 ? end - start : 1;
    h_mv_make(&G.V_tmp, n, width, NULL);
    G.sub_dtmp = (double *)calloc((size_t)(ncols + 1) * (ncols + 1) + 64, sizeof(double));
    /* the column handles may be permuted by zero-vector swaps: copy back in order */
    int new_end = stable_multi_orth(&G, &V, start, end, B_rp ? &Bm : NULL);
    double *tmp = (double *)malloc(sizeof(double) * (size_t)n * ncols);
    for (int j = 0; j < ncols; ++j) memcpy(tmp + (size_t)j * n, hcol(V.c[j]), sizeof(double) * n);
    memcpy(Vd, tmp, sizeof(double) * (size_t)n * ncols);
    free(tmp);
    h_mv_free(&G.V_tmp);
    free(G.sub_dtmp);
    h_mv_free(&V);
    return new_end;
}

/* ------------------------------------------- table-driven solve: helpers */
size_t gcge_oracle_table_bytes(void) { return sizeof(ops_t); }

void gcge_oracle_host_table(void *table) { memcpy(table, &H_OPS, sizeof(ops_t)); }

void *gcge_oracle_csr_handle(int n, const int *rp, const int *ci, const double *v)
{
    csr_t *A = (csr_t *)malloc(sizeof(csr_t));
    A->n = n; A->rp = rp; A->ci = ci; A->v = v;
    return A;
}
void gcge_oracle_csr_handle_free(void *A) { free(A); }

int gcge_oracle_table_mv_create(void *table, void *mat, int k, void ***mv)
{
    ops_t *ops = (ops_t *)table;
    *mv = NULL;
    if (!ops || !ops->MultiVecCreateByMat || !mat || k <= 0) return 1;
    ops->MultiVecCreateByMat(mv, k, mat, ops);
    return *mv ? 0 : 1;
}
void gcge_oracle_table_mv_destroy(void *table, void ***mv, int k)
{
    ops_t *ops = (ops_t *)table;
    if (ops && ops->MultiVecDestroy && mv && *mv) ops->MultiVecDestroy(mv, k, ops);
}
void gcge_oracle_host_mv_read(void **mv, int k, int n, double *out)
{
    for (int j = 0; j < k; ++j) memcpy(out + (size_t)j * n, hcol(mv[j]), sizeof(double) * n);
}

/* ------------------------------------------------ double-double checkers */
/* Error-free transformations (Knuth's TwoSum, the fused multiply-add form of
 * TwoProduct; Dekker, Numer. Math. 18, 1971) and double-double sums, used by the
 * finite-difference check of the gradients: eigenvalues of a perturbed problem
 * as Rayleigh quotients and eigenvectors refined by one correction step, both
 * far more accurate than one FP64 rounding of the loss. Not a reference
 * restatement: checker arithmetic only. */
typedef struct { double hi, lo; } dd_t;

static void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b, bv = x - a, av = x - bv;
    *s = x;
    *e = (a - av) + (b - bv);
}
static dd_t dd_norm(double s, double e)
{
    dd_t r;
    r.hi = s + e;
    r.lo = e - (r.hi - s);
    return r;
}
static dd_t dd_add(dd_t a, dd_t b)
{
    double s, e;
    two_sum(a.hi, b.hi, &s, &e);
    return dd_norm(s, e + (a.lo + b.lo));
}
static dd_t dd_prod(double a, double b)
{
    dd_t r;
    r.hi = a * b;
    r.lo = fma(a, b, -r.hi);
    return r;
}
static dd_t dd_mul(dd_t a, dd_t b)
{
    dd_t p = dd_prod(a.hi, b.hi);
    return dd_norm(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
static dd_t dd_div(dd_t a, dd_t b)
{
    double q1 = a.hi / b.hi;
    dd_t r = dd_add(a, dd_mul(b, (dd_t){-q1, 0.0}));
    double q2 = r.hi / b.hi;
    r = dd_add(r, dd_mul(b, (dd_t){-q2, 0.0}));
    double q3 = r.hi / b.hi;
    dd_t q = dd_norm(q1, q2);
    return dd_add(q, (dd_t){q3, 0.0});
}
/* (A x)_i with x = xh + xl, in double-double */
static dd_t dd_row(const int *rp, const int *ci, const double *v, int i, const double *xh, const double *xl)
{
    dd_t y = {0.0, 0.0};
    for (int j = rp[i]; j < rp[i + 1]; ++j) {
        y = dd_add(y, dd_prod(v[j], xh[ci[j]]));
        if (xl) y = dd_add(y, dd_prod(v[j], xl[ci[j]]));
    }
    return y;
}

/* out[0..1] = (x^T A x) / (x^T x) in double-double, x = xh + xl (xl may be NULL) */
void gcge_oracle_dd_rayleigh(int n, const int *rp, const int *ci, const double *v, const double *xh,
                             const double *xl, double *out)
{
    dd_t xax = {0.0, 0.0}, xx = {0.0, 0.0};
    for (int i = 0; i < n; ++i) {
        dd_t xi = {xh[i], xl ? xl[i] : 0.0};
        xax = dd_add(xax, dd_mul(dd_row(rp, ci, v, i, xh, xl), xi));
        xx = dd_add(xx, dd_mul(xi, xi));
    }
    dd_t q = dd_div(xax, xx);
    out[0] = q.hi;
    out[1] = q.lo;
}

/* r = A x - theta x, formed in double-double and rounded once per entry */
void gcge_oracle_dd_residual(int n, const int *rp, const int *ci, const double *v, const double *xh,
                             const double *xl, double th_hi, double th_lo, double *r)
{
    dd_t th = {-th_hi, -th_lo};
    for (int i = 0; i < n; ++i) {
        dd_t xi = {xh[i], xl ? xl[i] : 0.0};
        dd_t y = dd_add(dd_row(rp, ci, v, i, xh, xl), dd_mul(th, xi));
        r[i] = y.hi + y.lo;
    }
}

/* x += d in double-double (x = xh + xl) */
void gcge_oracle_dd_add_vec(int n, double *xh, double *xl, const double *d)
{
    for (int i = 0; i < n; ++i) {
        dd_t x = dd_add((dd_t){xh[i], xl[i]}, (dd_t){d[i], 0.0});
        xh[i] = x.hi;
        xl[i] = x.lo;
    }
}

/* out[0..3] = sum_i w_i x_i^2 and sum_i x_i^2 in double-double, x = xh + xl */
void gcge_oracle_dd_weighted_sq(int n, const double *w, const double *xh, const double *xl, double *out)
{
    dd_t s = {0.0, 0.0}, t = {0.0, 0.0};
    for (int i = 0; i < n; ++i) {
        dd_t xi = {xh[i], xl ? xl[i] : 0.0};
        dd_t x2 = dd_mul(xi, xi);
        s = dd_add(s, dd_mul(x2, (dd_t){w[i], 0.0}));
        t = dd_add(t, x2);
    }
    out[0] = s.hi; out[1] = s.lo; out[2] = t.hi; out[3] = t.lo;
}
