/*
 * gb_ops_table.c -- device implementations behind the GCGE_OPS plug-in table
 * (src/gcge_ops.h:29-215), installed by GCGE_GPU_SetOps.
 *
 * A vector handle names one column of a row-major device block; a multivector
 * handle array names consecutive columns of one block, so every multivector
 * member is a single block kernel over a column range. Members keep the
 * reference's void signatures and record failures on the bound context.
 */
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gb_internal.h"
#include "gb_orth.h"
#include "gcge_gb300_ops.h"

typedef struct {
    gcge_gpu_mv *mv;   /* block the vector lives in */
    int col;           /* its column */
    int owner;         /* 1: this handle owns the block */
} gvec;

static gcge_gpu_ctx *g_ctx = NULL;
static unsigned long long g_seed = 1, g_draw = 0;

static gvec *H(void *p) { return (gvec *)p; }
static double *colptr(const gvec *v) { return v->mv->d + v->col; }

static void rec(int st)
{
    if (st && g_ctx) gb_fail(g_ctx, st);
}

void GCGE_GPU_OpsSeed(unsigned long long seed)
{
    g_seed = seed;
    g_draw = 0;
}

static gvec *vnew(gcge_gpu_mv *mv, int col, int owner)
{
    gvec *v = (gvec *)malloc(sizeof(gvec));
    if (!v) return NULL;
    v->mv = mv;
    v->col = col;
    v->owner = owner;
    return v;
}

/* ---------------------------------------------------------- single vectors */
static void op_vec_create_by_n(void **vec, int n)
{
    gcge_gpu_mv *mv = NULL;
    int st = GCGE_GPU_MultiVecCreate(g_ctx, n, 1, &mv);
    if (st) { rec(st); *vec = NULL; return; }
    *vec = vnew(mv, 0, 1);
}
static void op_VecCreateByMat(void **vec, void *mat) { op_vec_create_by_n(vec, ((gcge_gpu_mat *)mat)->n); }
static void op_VecCreateByVec(void **des, void *src) { op_vec_create_by_n(des, H(src)->mv->n); }
static void op_VecDestroy(void **vec)
{
    if (!vec || !*vec) return;
    gvec *v = H(*vec);
    if (v->owner) GCGE_GPU_MultiVecDestroy(v->mv);
    free(v);
    *vec = NULL;
}
static void op_VecSetRandomValue(void *vec)
{
    gvec *v = H(vec);
    rec(gb_fill_random(g_ctx, v->mv->n, 1, colptr(v), v->mv->ld, (int)(g_draw++), g_seed));
}
static void op_MatDotVec(void *mat, void *x, void *r)
{
    gcge_gpu_mat *A = (gcge_gpu_mat *)mat;
    rec(gb_spmm(g_ctx, A, colptr(H(x)), H(x)->mv->ld, colptr(H(r)), H(r)->mv->ld, 1, 1.0, NULL, 0.0, NULL));
}
static void op_VecAxpby(double a, void *x, double b, void *y)
{
    rec(gb_axpby(g_ctx, H(y)->mv->n, 1, a, colptr(H(x)), H(x)->mv->ld, b, colptr(H(y)), H(y)->mv->ld));
}
static void op_VecInnerProd(void *x, void *y, double *value)
{
    int st = gb_coef(g_ctx, 8);
    if (!st) st = gb_col_dots(g_ctx, H(x)->mv->n, 1, colptr(H(x)), H(x)->mv->ld, colptr(H(y)), H(y)->mv->ld, g_ctx->coef);
    if (!st && (cudaMemcpyAsync(value, g_ctx->coef, sizeof(double), cudaMemcpyDeviceToHost, g_ctx->stream) != cudaSuccess ||
                cudaStreamSynchronize(g_ctx->stream) != cudaSuccess))
        st = GCGE_GPU_ERR_CUDA;
    rec(st);
}

/* ---------------------------------------------------------- multivectors */
static void op_mv_create_n(void ***mv, int n_vec, int n)
{
    gcge_gpu_mv *blk = NULL;
    *mv = NULL;
    int st = GCGE_GPU_MultiVecCreate(g_ctx, n, n_vec > 0 ? n_vec : 1, &blk);
    if (st) { rec(st); return; }
    void **h = (void **)malloc(sizeof(void *) * (n_vec > 0 ? n_vec : 1));
    if (!h) { GCGE_GPU_MultiVecDestroy(blk); rec(GCGE_GPU_ERR_NOMEM); return; }
    for (int i = 0; i < n_vec; ++i) h[i] = vnew(blk, i, i == 0);
    *mv = h;
}
static void op_MultiVecCreateByMat(void ***mv, int n_vec, void *mat, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    op_mv_create_n(mv, n_vec, ((gcge_gpu_mat *)mat)->n);
}
static void op_MultiVecCreateByVec(void ***mv, int n_vec, void *vec, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    op_mv_create_n(mv, n_vec, H(vec)->mv->n);
}
static void op_MultiVecCreateByMultiVec(void ***mv, int n_vec, void **init, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    op_mv_create_n(mv, n_vec, H(init[0])->mv->n);
}
static void op_MultiVecDestroy(void ***mv, int n_vec, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    if (!mv || !*mv) return;
    void **h = *mv;
    gcge_gpu_mv *blk = n_vec > 0 && h[0] ? H(h[0])->mv : NULL;
    for (int i = 0; i < n_vec; ++i) free(h[i]);
    if (blk) GCGE_GPU_MultiVecDestroy(blk);
    free(h);
    *mv = NULL;
}

/* resolve a column range [s, s+k) of a handle array to (block, first column);
 * 0 when the handles are not consecutive columns of one block */
static int resolve(void **h, int s, int k, gcge_gpu_mv **blk, int *c0)
{
    if (k <= 0) { *blk = H(h[s > 0 ? 0 : 0])->mv; *c0 = 0; return 1; }
    gvec *a = H(h[s]), *b = H(h[s + k - 1]);
    if (a->mv != b->mv || b->col != a->col + k - 1) return 0;
    *blk = a->mv;
    *c0 = a->col;
    return 1;
}

int GCGE_GPU_OpsMultiVecBlock(void **multi_vec, gcge_gpu_mv **block, int *first_col)
{
    if (!multi_vec || !multi_vec[0] || !block || !first_col) return GCGE_GPU_ERR_ARG;
    *block = H(multi_vec[0])->mv;
    *first_col = H(multi_vec[0])->col;
    return GCGE_GPU_OK;
}

static void op_MultiVecSetRandomValue(void **mv, int start, int n_vec, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    for (int i = 0; i < n_vec; ++i) op_VecSetRandomValue(mv[start + i]);
}
static void op_MatDotMultiVec(void *mat, void **x, void **y, int *start, int *end, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    const int k = end[0] - start[0];
    gcge_gpu_mv *xb, *yb;
    int xc, yc;
    if (k <= 0) return;
    if (resolve(x, start[0], k, &xb, &xc) && resolve(y, start[1], k, &yb, &yc)) {
        gcge_gpu_mat *A = (gcge_gpu_mat *)mat;
        rec(gb_spmm(g_ctx, A, xb->d + xc, xb->ld, yb->d + yc, yb->ld, k, 1.0, NULL, 0.0, NULL));
    } else {
        for (int i = 0; i < k; ++i) op_MatDotVec(mat, x[start[0] + i], y[start[1] + i]);
    }
}
static void op_MultiVecAxpby(double a, void **x, double b, void **y, int *start, int *end, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    const int k = end[0] - start[0];
    gcge_gpu_mv *xb, *yb;
    int xc, yc;
    if (k <= 0) return;
    if (resolve(x, start[0], k, &xb, &xc) && resolve(y, start[1], k, &yb, &yc))
        rec(gb_axpby(g_ctx, xb->n, k, a, xb->d + xc, xb->ld, b, yb->d + yc, yb->ld));
    else
        for (int i = 0; i < k; ++i) op_VecAxpby(a, x[start[0] + i], b, y[start[1] + i]);
}
static void op_MultiVecAxpbyColumn(double a, void **x, int cx, double b, void **y, int cy, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    op_VecAxpby(a, x[cx], b, y[cy]);
}
static void op_MultiVecLinearComb(void **x, void **y, int *start, int *end, double *a, int lda, void *dmat, int lddmat,
                                  GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    (void)dmat;
    (void)lddmat;
    gcge_gpu_mv *xb, *yb;
    int xc, yc;
    const int k1 = end[0] - start[0], k2 = end[1] - start[1];
    if (k2 <= 0) return;
    if (!resolve(x, start[0], k1, &xb, &xc) || !resolve(y, start[1], k2, &yb, &yc)) { rec(GCGE_GPU_ERR_ARG); return; }
    int s[2] = {xc, yc}, e[2] = {xc + k1, yc + k2};
    rec(GCGE_GPU_MultiVecLinearComb(xb, yb, s, e, a, lda));
}
static void op_MultiVecInnerProd(void **V, void **W, double *a, char *is_sym, int *start, int *end, int lda,
                                 GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    gcge_gpu_mv *vb, *wb;
    int vc, wc;
    const int k1 = end[0] - start[0], k2 = end[1] - start[1];
    if (k1 <= 0 || k2 <= 0) return;
    if (!resolve(V, start[0], k1, &vb, &vc) || !resolve(W, start[1], k2, &wb, &wc)) { rec(GCGE_GPU_ERR_ARG); return; }
    int s[2] = {vc, wc}, e[2] = {vc + k1, wc + k2};
    rec(GCGE_GPU_MultiVecInnerProd(vb, wb, a, is_sym, s, e, lda));
}
static void op_MultiVecSwap(void **V1, void **V2, int *start, int *end, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    const int k = end[0] - start[0];
    if (k <= 0) return;
    for (int i = 0; i < k; ++i) {
        gvec *a = H(V1[start[0] + i]), *b = H(V2[start[1] + i]);
        int s[2] = {a->col, b->col}, e[2] = {a->col + 1, b->col + 1};
        if (a == b) continue;
        if (i == 0) {
            /* whole range at once when both sides are consecutive */
            gcge_gpu_mv *xb, *yb;
            int xc, yc;
            if (resolve(V1, start[0], k, &xb, &xc) && resolve(V2, start[1], k, &yb, &yc) &&
                (xb != yb || xc + k <= yc || yc + k <= xc)) {
                int s2[2] = {xc, yc}, e2[2] = {xc + k, yc + k};
                rec(GCGE_GPU_MultiVecSwap(xb, yb, s2, e2));
                return;
            }
        }
        rec(GCGE_GPU_MultiVecSwap(a->mv, b->mv, s, e));
    }
}
static void op_MultiVecPrint(void **x, int n)
{
    for (int i = 0; i < n; ++i) {
        gvec *v = H(x[i]);
        double *h = (double *)malloc(sizeof(double) * v->mv->n);
        if (!h) return;
        if (!gb_download_cols(g_ctx, v->mv->n, 1, colptr(v), v->mv->ld, h)) {
            printf("num size = %d\n", v->mv->n);
            for (int r = 0; r < v->mv->n; ++r) printf("%0.4f\t", h[r]);
            printf("\n");
        }
        free(h);
    }
}
static void op_GetVecFromMultiVec(void **V, int j, void **x) { *x = V[j]; }
static void op_RestoreVecForMultiVec(void **V, int j, void **x) { V[j] = *x; }
static void op_SetDirichletBoundary(void **Vecs, int nev, void *A, void *B)
{
    gcge_gpu_mv *blk;
    int c0;
    if (nev <= 0 || !A || !B) return;
    if (resolve(Vecs, 0, nev, &blk, &c0))
        rec(gb_dirichlet_zero(g_ctx, (gcge_gpu_mat *)A, (gcge_gpu_mat *)B, nev, blk->d + c0, blk->ld));
    else
        for (int i = 0; i < nev; ++i)
            rec(gb_dirichlet_zero(g_ctx, (gcge_gpu_mat *)A, (gcge_gpu_mat *)B, 1, colptr(H(Vecs[i])), H(Vecs[i])->mv->ld));
}

/* dsyevx-signature eigensolve (jobz "V", range "I", uplo "U") on the device */
static void op_DenseMatEigenSolver(char *jobz, char *range, char *uplo, int *nrows, double *a, int *lda, double *vl,
                                   double *vu, int *il, int *iu, double *abstol, int *nev, double *eval, double *evec,
                                   int *lde, int *isuppz, double *work, int *lwork, int *iwork, int *liwork, int *ifail,
                                   int *info)
{
    (void)vl; (void)vu; (void)abstol; (void)isuppz; (void)work; (void)lwork; (void)iwork; (void)liwork; (void)ifail;
    const int m = *nrows, lo = *il, hi = *iu, k = hi - lo + 1;
    *info = 0;
    if (jobz[0] != 'V' || range[0] != 'I' || uplo[0] != 'U' || m <= 0 || lo < 1 || hi > m || lo > hi) {
        *info = -1;
        rec(GCGE_GPU_ERR_ARG);
        return;
    }
    double *dH = NULL, *dZ = NULL, *dE = NULL, *dW = NULL;
    int *dInfo = NULL, hinfo = 0, st = 0;
    if (cudaMalloc((void **)&dH, sizeof(double) * (size_t)m * m) != cudaSuccess ||
        cudaMalloc((void **)&dZ, sizeof(double) * (size_t)m * k) != cudaSuccess ||
        cudaMalloc((void **)&dE, sizeof(double) * (size_t)m) != cudaSuccess ||
        cudaMalloc((void **)&dW, sizeof(double) * gb_syevx_work_doubles(m)) != cudaSuccess ||
        cudaMalloc((void **)&dInfo, sizeof(int) * 2) != cudaSuccess)
        st = GCGE_GPU_ERR_NOMEM;
    if (!st && cudaMemcpy2DAsync(dH, sizeof(double) * m, a, sizeof(double) * (*lda), sizeof(double) * m, m,
                                 cudaMemcpyHostToDevice, g_ctx->stream) != cudaSuccess)
        st = GCGE_GPU_ERR_CUDA;
    if (!st) st = gb_symmetrize_from_upper(g_ctx, dH, m, m);
    if (!st) st = gb_syevx(g_ctx, m, dH, m, lo, hi, dE, dZ, m, dW, dInfo);
    if (!st && (cudaMemcpyAsync(eval, dE, sizeof(double) * k, cudaMemcpyDeviceToHost, g_ctx->stream) != cudaSuccess ||
                cudaMemcpy2DAsync(evec, sizeof(double) * (*lde), dZ, sizeof(double) * m, sizeof(double) * m, k,
                                  cudaMemcpyDeviceToHost, g_ctx->stream) != cudaSuccess ||
                cudaMemcpyAsync(&hinfo, dInfo, sizeof(int), cudaMemcpyDeviceToHost, g_ctx->stream) != cudaSuccess))
        st = GCGE_GPU_ERR_CUDA;
    if (cudaStreamSynchronize(g_ctx->stream) != cudaSuccess) st = GCGE_GPU_ERR_CUDA;
    if (!st && hinfo) st = GCGE_GPU_ERR_EIGSOLVE;
    cudaFree(dH); cudaFree(dZ); cudaFree(dE); cudaFree(dW); cudaFree(dInfo);
    *nev = k;
    if (st) *info = 1;
    rec(st);
}

/* ---------------------------------------------------------- LinearSolver hook */
/* The reference calls ops->LinearSolver(A, b, x, ops) once per W column in place of
 * its block CG (src/gcge_xpw.c:177-191); its parameters cannot travel through that
 * signature, so they are set here. Kind 1: Jacobi-preconditioned CG on the device
 * (the block CG of this library with k = 1 and z = diag(A)^-1 r) from the given x,
 * to ||r||_z <= rate ||r0||_z or max_it iterations; b is left unchanged. */
static int g_ls_max_it = 20;
static double g_ls_rate = 1e-2;
static gcge_gpu_mv *g_ls_rhs = NULL;     /* copy of b (the block CG overwrites its right-hand side) */
static void *g_ls_work = NULL;
static size_t g_ls_work_bytes = 0;

static void op_LinearSolverJacobi(void *mat, void *b, void *x, GCGE_GPU_OPS_LAYOUT *ops)
{
    (void)ops;
    gcge_gpu_mat *A = (gcge_gpu_mat *)mat;
    gvec *vb = H(b), *vx = H(x);
    const int n = A->n;
    int st = 0;
    if (!g_ctx || vb->mv->n != n || vx->mv->n != n) {
        rec(GCGE_GPU_ERR_ARG);
        return;
    }
    if (g_ls_rhs && g_ls_rhs->n != n) {
        GCGE_GPU_MultiVecDestroy(g_ls_rhs);
        g_ls_rhs = NULL;
    }
    if (!g_ls_rhs && (st = GCGE_GPU_MultiVecCreate(g_ctx, n, 1, &g_ls_rhs))) {
        rec(st);
        return;
    }
    const size_t need = gb_bcg_work_bytes(n, 1, 0);
    if (need > g_ls_work_bytes) {
        cudaFree(g_ls_work);
        g_ls_work = NULL;
        g_ls_work_bytes = 0;
        if (cudaMalloc(&g_ls_work, need) != cudaSuccess) {
            rec(GCGE_GPU_ERR_NOMEM);
            return;
        }
        g_ls_work_bytes = need;
    }
    if ((st = gb_mat_dinv(g_ctx, A))) {
        rec(st);
        return;
    }
    if ((st = gb_axpby(g_ctx, n, 1, 1.0, colptr(vb), vb->mv->ld, 0.0, g_ls_rhs->d, g_ls_rhs->ld))) {
        rec(st);
        return;
    }
    gb_bcg_args a;
    memset(&a, 0, sizeof(a));
    a.n = n;
    a.k = 1;
    a.max_it = g_ls_max_it;
    a.precision = 0;
    a.rate = g_ls_rate;
    a.dinv = A->dinv;
    a.dinv32 = A->dinv32;
    rec(gb_bcg(g_ctx, A, g_ls_rhs->d, g_ls_rhs->ld, colptr(vx), vx->mv->ld, &a, g_ls_work, g_ls_work_bytes));
}

int GCGE_GPU_OpsSetLinearSolver(void *gcge_ops, int kind, int max_it, double rate)
{
    if (!gcge_ops || kind < 0 || kind > 1 || max_it < 1 || !(rate > 0)) return GCGE_GPU_ERR_ARG;
    GCGE_GPU_OPS_LAYOUT *ops = (GCGE_GPU_OPS_LAYOUT *)gcge_ops;
    g_ls_max_it = max_it;
    g_ls_rate = rate;
    ops->LinearSolver = kind == 1 ? op_LinearSolverJacobi : NULL;
    return GCGE_GPU_OK;
}

int GCGE_GPU_SetOps(gcge_gpu_ctx *ctx, void *table)
{
    if (!ctx || !table) return GCGE_GPU_ERR_ARG;
    GCGE_GPU_OPS_LAYOUT *ops = (GCGE_GPU_OPS_LAYOUT *)table;
    g_ctx = ctx;
    ops->VecSetRandomValue = op_VecSetRandomValue;
    ops->MatDotVec = op_MatDotVec;
    ops->VecAxpby = op_VecAxpby;
    ops->VecInnerProd = op_VecInnerProd;
    ops->VecLocalInnerProd = op_VecInnerProd;
    ops->VecCreateByVec = op_VecCreateByVec;
    ops->VecCreateByMat = op_VecCreateByMat;
    ops->VecDestroy = op_VecDestroy;
    ops->MultiVecCreateByVec = op_MultiVecCreateByVec;
    ops->MultiVecCreateByMat = op_MultiVecCreateByMat;
    ops->MultiVecCreateByMultiVec = op_MultiVecCreateByMultiVec;
    ops->MultiVecDestroy = op_MultiVecDestroy;
    ops->MultiVecSetRandomValue = op_MultiVecSetRandomValue;
    ops->MatDotMultiVec = op_MatDotMultiVec;
    ops->MultiVecAxpby = op_MultiVecAxpby;
    ops->MultiVecAxpbyColumn = op_MultiVecAxpbyColumn;
    ops->MultiVecLinearComb = op_MultiVecLinearComb;
    ops->MultiVecInnerProd = op_MultiVecInnerProd;
    ops->MultiVecSwap = op_MultiVecSwap;
    ops->MultiVecPrint = op_MultiVecPrint;
    ops->GetVecFromMultiVec = op_GetVecFromMultiVec;
    ops->RestoreVecForMultiVec = op_RestoreVecForMultiVec;
    ops->SetDirichletBoundary = op_SetDirichletBoundary;
    ops->DenseMatEigenSolver = op_DenseMatEigenSolver;
    return GCGE_GPU_OK;
}
