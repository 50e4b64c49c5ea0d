/*
 * gb_solver.c -- the GCG eigensolver driver on one GB300 (host side, C).
 *
 * Control flow, index bookkeeping and parameter semantics follow GCGE_Solve
 * (src/gcge_eigsol.c:65-542) phase by phase: initial X, Rayleigh-Ritz on X, W
 * from block CG, [X,W] step, then the [X,P,W] loop with CheckEvalMultiplicity
 * and CheckConvergence. What differs is where the data lives and how each
 * phase is computed:
 *   - every n-sized block (V = [X,P,W], the Ritz vectors, scratch) is a row-
 *     major block in HBM, and every small dense matrix (projected matrix H,
 *     coefficients C, Gram blocks) stays in device memory;
 *   - W is B-orthonormalised by block projection + Cholesky-QR twice
 *     (gb_orthonormalize) instead of the recursive block Gram-Schmidt;
 *   - the projected eigenproblem is solved on the device (gb_syevx);
 *   - block CG keeps its per-column state on the device (gb_bcg), optionally in
 *     FP32 (mixed precision);
 *   - one small device-to-host copy per iteration (eigenvalues and residual
 *     norms) feeds the host-side convergence and multiplicity logic, plus one
 *     per Cholesky-QR pass (the kept-column count).
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gb_internal.h"
#include "gb_orth.h"

int gb_select(gcge_gpu_ctx *ctx, int k, const double *src, const int *idx, double *out);
int gb_scale_cols(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const double *s, double *Y, long ldy);

#define TRY(x)                  \
    do {                        \
        int _s = (x);           \
        if (_s) { st = _s; goto fail; } \
    } while (0)
#define CTRY(x)                                          \
    do {                                                 \
        if ((x) != cudaSuccess) { st = gb_fail(ctx, GCGE_GPU_ERR_CUDA); goto fail; } \
    } while (0)

enum { PH_X_AXPY, PH_X_ORTH, PH_P_AXPY, PH_P_ORTH, PH_W_LINE, PH_W_ORTH, PH_RR_MAT, PH_RR_EIGEN, PH_CONV, PH_N };

typedef struct {
    cudaEvent_t ev[2 * 64];
    int slot[64];
    int used;
    double ms[PH_N];
} phase_timer;

typedef struct {
    gcge_gpu_ctx *ctx;
    const gcge_gpu_mat *A, *B;
    gcge_gpu_params p;
    int n, nev, bs, max_dim_x, V_size, S_width;
    /* device blocks */
    double *V, *X, *S1, *S2, *S3;
    long ldv, ldx, lds;
    void *bcg_work;
    size_t bcg_bytes;
    /* device small dense */
    double *H, *C, *Ctmp, *AApp, *Gs, *Ts, *chol_work, *eval_d, *eig_work, *res_d, *lam_d, *dsmall, *nu_d;
    int *unlock_d, *kept_d, *info_d, *pos_d;
    /* host */
    double *eval_h, *res_h, *resv;
    int *unlock_h, *pos_h;
    /* S2 = A X and S3 = B X for the unlock list the last convergence check saw;
     * pos_h[j] = position of the j-th unlocked column in that list */
    int conv_products;
    /* state (GCGE_WORKSPACE / GCGE_PARA members) */
    int dim_x, dim_xp, dim_xpw, last_dim_xpw, last_dim_x, unconv_bs, num_unlock, num_iter;
    double max_res, min_res, sum_res, conv_omega_norm, zero_tol;
    int orth_kind;             /* w_orth_type variant (gb_orth.h) */
    int amode;                 /* orth_type "A": basis A-orthonormal, projected matrix -V^T B V */
    const gcge_gpu_mat *Om;    /* the orthonormalisation matrix: B, or A in A-orthogonal mode */
    int soft_locked;           /* Ritz pairs soft-locked in the last Rayleigh-Ritz step */
    gb_orth_ws ows;
    phase_timer tm;
} gcg_t;

static int d2h(gcge_gpu_ctx *ctx, void *dst, const void *src, size_t bytes)
{
    if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    return 0;
}
static int h2d(gcge_gpu_ctx *ctx, void *dst, const void *src, size_t bytes)
{
    if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    return 0;
}

static void ph_begin(gcg_t *g, int slot)
{
    phase_timer *t = &g->tm;
    if (t->used >= 64) return;
    t->slot[t->used] = slot;
    cudaEventRecord(t->ev[2 * t->used], g->ctx->stream);
}
static void ph_end(gcg_t *g)
{
    phase_timer *t = &g->tm;
    if (t->used >= 64) return;
    cudaEventRecord(t->ev[2 * t->used + 1], g->ctx->stream);
    t->used++;
}
/* with no interval open: wait for the last one, fold the intervals into the totals */
static void ph_collect(gcg_t *g)
{
    phase_timer *t = &g->tm;
    if (t->used > 0) cudaEventSynchronize(t->ev[2 * t->used - 1]);
    for (int i = 0; i < t->used; ++i) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, t->ev[2 * i], t->ev[2 * i + 1]) == cudaSuccess) t->ms[t->slot[i]] += ms;
    }
    t->used = 0;
}

void GCGE_GPU_ParamsDefault(gcge_gpu_params *p)
{
    memset(p, 0, sizeof(*p));
    p->nev = 1;
    p->block_size = 0;
    p->ev_max_it = 30;
    p->cg_max_it = 20;
    p->max_reorth_time = 3;
    p->ev_tol = 1e-8;
    p->cg_rate = 1e-2;
    p->orth_zero_tol = 1e-16;
    strcpy(p->conv_type, "R");
    strcpy(p->w_orth_type, "multi");
    p->opt_rr_eig_partly = 0;
    p->multi_tol_for_lock = 1e-6;
    strcpy(p->orth_type, "B");
    p->precision = 0;
    p->seed = 1;
}

/* ------------------------------------------------------------ Rayleigh-Ritz */
/* GCGE_ComputeSubspaceMatrix (src/gcge_rayleighritz.c:113-200): XAX = diag(eval),
 * XAP = 0, PAP = pp^T H_old pp, then [X,P,W]^T A W from one SpMM and two Grams;
 * H is kept fully symmetric (upper triangle mirrored). In A-orthogonal mode the
 * basis is A-orthonormal and H = -V^T B V, whose smallest eigenvalues nu are
 * the largest of V^T B V (lambda = -1/nu): its X block is diag(nu) of the last
 * step and its W columns come from -B W. */
static int rr_matrix(gcg_t *g)
{
    gcge_gpu_ctx *ctx = g->ctx;
    int st = 0;
    const int dim_xp = g->dim_xp, ldm = g->dim_xpw, n = g->n;
    if (dim_xp != 0) {
        const int lde = g->last_dim_xpw, dim_x = g->dim_x, dim_p = dim_xp - dim_x;
        const double *pp = g->C + (size_t)dim_x * lde;
        if (dim_p > 0)
            TRY(gb_small_gemm(ctx, 'N', 'N', lde, dim_p, lde, 1.0, g->H, lde, pp, lde, 0.0, g->AApp, lde));
        TRY(gb_set_zero(ctx, g->H, (size_t)ldm * ldm));
        if (dim_p > 0)
            TRY(gb_small_gemm(ctx, 'T', 'N', dim_p, dim_p, lde, 1.0, pp, lde, g->AApp, lde, 0.0,
                              g->H + (size_t)dim_x * ldm + dim_x, ldm));
        TRY(gb_set_diag_from(ctx, g->H, ldm, dim_x, g->amode ? g->nu_d : g->eval_d));
    }
    /* VTAW (src/gcge_rayleighritz.c:35-81): AW = A W into S1 (A-orthogonal mode: -B W) */
    const int w_len = ldm - dim_xp, xp_len = dim_xp;
    if (!g->amode)
        TRY(gb_spmm(ctx, g->A, g->V + dim_xp, g->ldv, g->S1, g->lds, w_len, 1.0, NULL, 0.0, NULL));
    else if (g->B)
        TRY(gb_spmm(ctx, g->B, g->V + dim_xp, g->ldv, g->S1, g->lds, w_len, -1.0, NULL, 0.0, NULL));
    else
        TRY(gb_axpby(ctx, n, w_len, -1.0, g->V + dim_xp, g->ldv, 0.0, g->S1, g->lds));
    /* [X P W]^T (A W) in one Gram: H[0:ldm, dim_xp:ldm] (the W^T A W block in full;
     * its lower half is then replaced by the mirrored upper half) */
    (void)xp_len;
    TRY(gb_gram(ctx, n, ldm, w_len, g->V, g->ldv, g->S1, g->lds, g->H + (size_t)dim_xp * ldm, ldm, 0));
    TRY(gb_symmetrize_from_upper(ctx, g->H, ldm, ldm));
    return 0;
fail:
    return st;
}

/* GCGE_ComputeSubspaceEigenpairs (src/gcge_rayleighritz.c:364-590) with
 * opt_rr_eig_partly = 0: eigenpairs 1 .. min(max_dim_x, ldm). In A-orthogonal
 * mode the eigenvalues nu of -V^T B V come out ascending; lambda = -1/nu keeps
 * that order (the reference solves V^T B V for its smallest eigenvalues and
 * reverses them with GCGE_SortEigenpairs, src/gcge_rayleighritz.c:581-617,
 * which picks the wrong end of its spectrum). */
static int rr_eig_solve(gcg_t *g);
static int rr_eig(gcg_t *g)
{
    const int ldm = g->dim_xpw, iu = g->max_dim_x < ldm ? g->max_dim_x : ldm;
    int st = rr_eig_solve(g);
    if (st || !g->amode) return st;
    const int s = g->soft_locked;
    return gb_neg_recip(g->ctx, iu - s, g->eval_d + s, g->nu_d + s);
}
static int rr_eig_solve(gcg_t *g)
{
    const int ldm = g->dim_xpw;
    const int iu = g->max_dim_x < ldm ? g->max_dim_x : ldm;
    int sl = 0;
    if (g->p.opt_rr_eig_partly && g->num_unlock > 0) {
        /* soft locking (src/gcge_rayleighritz.c:378-394): the first unconverged
         * index, lowered by every earlier eigenvalue within multi_tol_for_lock */
        const int s0 = g->unlock_h[0];
        sl = s0;
        for (int i = s0 - 1; i >= 0; --i)
            if (fabs(g->eval_h[i] - g->eval_h[s0]) / g->eval_h[s0] < g->p.multi_tol_for_lock) sl -= 1;
        if (sl < 0) sl = 0;
        if (sl > g->dim_x) sl = g->dim_x;
        if (sl >= iu) sl = 0;
    }
    g->soft_locked = sl;
    /* the previous step's eigenvalues of the projected matrix start the bisection
     * (lambda, or nu in A-orthogonal mode; zeros before the first step) */
    const double *guess = g->amode ? g->nu_d : g->eval_d;
    if (sl == 0)
        return gb_syevx_guess(g->ctx, ldm, g->H, ldm, 1, iu, g->eval_d, g->C, ldm, g->eig_work, g->info_d, guess);
    /* the locked pairs keep their eigenvalues and are the unit vectors of the
     * projected basis; only the trailing (ldm - sl) block is solved */
    int st = gb_soft_lock(g->ctx, g->H, ldm, ldm, g->dim_xp, sl, g->C, ldm, iu);
    if (st) return st;
    return gb_syevx_guess(g->ctx, ldm - sl, g->H + (size_t)sl * ldm + sl, ldm, 1, iu - sl, g->eval_d + sl,
                          g->C + (size_t)sl * ldm + sl, ldm, g->eig_work, g->info_d, guess + sl);
}

/* GCGE_ComputeX (src/gcge_xpw.c:47-76): X[:, s:nev] = V[:, s:dim_xpw] C[s:, s:nev], s
 * the soft-locked count (0 without soft locking; the locked columns are unchanged) */
static int compute_x(gcg_t *g)
{
    const int s = g->soft_locked;
    if (s >= g->nev) return 0;
    return gb_lincomb(g->ctx, g->n, g->dim_xpw - s, g->nev - s, g->V + s, g->ldv, g->C + (size_t)s * g->dim_xpw + s,
                      g->dim_xpw, 1.0, 0.0, g->X + s, g->ldx, 0);
}

/* V[:, 0:nev] = X[:, 0:nev]: the pointer exchange of src/gcge_eigsol.c:312/417 as
 * a one-way copy (the old V columns are only scratch afterwards) */
static int x_to_v(gcg_t *g) { return gb_axpby(g->ctx, g->n, g->nev, 1.0, g->X, g->ldx, 0.0, g->V, g->ldv); }

/* GCGE_CheckConvergence (src/gcge_eigsol.c:559-686): residuals of the columns in
 * the unlock list computed on the device in one batch; the reference's walk
 * (the "8 beyond the last converged" cut) is applied on the host. */
static int check_conv(gcg_t *g)
{
    gcge_gpu_ctx *ctx = g->ctx;
    int st = 0;
    const int nu = g->num_unlock, n = g->n;
    if (nu > 0) {
        CTRY(cudaMemcpyAsync(g->unlock_d, g->unlock_h, sizeof(int) * nu, cudaMemcpyHostToDevice, ctx->stream));
        /* the unlocked columns are usually a contiguous range of X (the trailing
         * unconverged pairs): then the products read X in place, else a gather */
        int contiguous = 1;
        for (int j = 1; j < nu; ++j)
            if (g->unlock_h[j] != g->unlock_h[0] + j) contiguous = 0;
        const double *Xu = g->S1;
        long ldu = g->lds;
        if (contiguous) {
            Xu = g->X + g->unlock_h[0];
            ldu = g->ldx;
        } else {
            TRY(gb_gather_cols(ctx, n, nu, g->X, g->ldx, g->unlock_d, g->S1, g->lds, NULL, 0));
        }
        TRY(gb_spmm_ab(ctx, g->A, g->B, Xu, ldu, g->S2, g->S3, g->lds, nu));
        TRY(gb_residual_norms(ctx, n, nu, Xu, ldu, g->S2, g->lds, g->B ? g->S3 : NULL, g->lds, g->eval_d,
                              g->unlock_d, g->res_d, strcmp(g->p.conv_type, "BR") == 0));
        CTRY(cudaMemcpyAsync(g->res_h, g->res_d, sizeof(double) * 3 * nu, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CTRY(cudaMemcpyAsync(g->eval_h, g->eval_d, sizeof(double) * g->V_size, cudaMemcpyDeviceToHost, ctx->stream));
    CTRY(cudaStreamSynchronize(ctx->stream));
    {
        int info = 0;
        TRY(d2h(ctx, &info, g->info_d, sizeof(int)));
        if (info) return gb_fail(ctx, GCGE_GPU_ERR_EIGSOLVE);
    }
    int unconv = 0, max_conv_idx = 0;
    double max_res = 0, min_res = 0, sum_res = 0;
    const char *ct = g->p.conv_type;
    for (int j = 0; j < nu; ++j) {
        const int i = g->unlock_h[j];
        const double lam = g->eval_h[i];
        const double rn = sqrt(g->res_h[3 * j]), en = sqrt(g->res_h[3 * j + 1]), bn = sqrt(g->res_h[3 * j + 2]);
        double r;
        if (!isfinite(rn) || !isfinite(en)) return gb_fail(ctx, GCGE_GPU_ERR_NONFINITE);
        if (strcmp(ct, "R") == 0) r = rn / en / (1.0 > fabs(lam) ? 1.0 : fabs(lam));
        else if (strcmp(ct, "O") == 0) r = rn / en / (g->conv_omega_norm + fabs(lam));
        else if (strcmp(ct, "BR") == 0) r = rn / (fabs(lam) * bn);
        else r = rn / en;
        g->resv[i] = r;
        sum_res += r;
        if (j == 0) { max_res = r; min_res = r; }
        else { if (r > max_res) max_res = r; if (r < min_res) min_res = r; }
        if (r > g->p.ev_tol) {
            g->pos_h[unconv] = j;
            g->unlock_h[unconv++] = i;
            if (j > max_conv_idx + 8) {
                for (int k = j + 1; k < nu; ++k) {
                    g->pos_h[unconv] = k;
                    g->unlock_h[unconv++] = g->unlock_h[k];
                }
                j = nu + 1;
            }
        } else {
            max_conv_idx = j;
        }
    }
    g->num_unlock = unconv;
    g->unconv_bs = unconv < g->bs ? unconv : g->bs;
    g->max_res = max_res;
    g->min_res = min_res;
    g->sum_res = sum_res;
    g->num_iter += 1;
    if (unconv > 0) {
        CTRY(cudaMemcpyAsync(g->unlock_d, g->unlock_h, sizeof(int) * unconv, cudaMemcpyHostToDevice, ctx->stream));
        CTRY(cudaMemcpyAsync(g->pos_d, g->pos_h, sizeof(int) * unconv, cudaMemcpyHostToDevice, ctx->stream));
        /* the copies read pos_h / unlock_h before the next host update: order them */
        CTRY(cudaStreamSynchronize(ctx->stream));
    }
    g->conv_products = nu > 0;
    if (g->p.print_level > 0)
        printf("num_unlock(%3d) = %3d; max_res(%3d) = %e; min_res(%3d) = %e;\n", g->num_iter, g->num_unlock,
               g->num_iter, max_res, g->num_iter, min_res);
    return 0;
fail:
    return st;
}

/* GCGE_ComputeW (src/gcge_xpw.c:118-217) + GCGE_BCG: initial guess x (|l| <= 1) or
 * x/l, right-hand side l B x (equivalently l B w in both cases) */
static int compute_w(gcg_t *g)
{
    gcge_gpu_ctx *ctx = g->ctx;
    int st = 0;
    const int ws = g->dim_xp, wl = g->unconv_bs, n = g->n;
    if (wl <= 0) return 0;
    double *W = g->V + ws;
    TRY(gb_gather_cols(ctx, n, wl, g->V, g->ldv, g->unlock_d, W, g->ldv, g->eval_d, 1));
    TRY(gb_select(ctx, wl, g->eval_d, g->unlock_d, g->lam_d));
    gb_bcg_args a;
    a.n = n;
    a.k = wl;
    a.max_it = g->p.cg_max_it;
    a.precision = g->p.precision;
    a.rate = g->p.cg_rate;
    a.rhs_is_residual = 0;
    a.dinv = NULL;
    a.dinv32 = NULL;
    a.residual_unused = 1;     /* S1 is scratch after the W step */
    if (g->p.precond == 1) {
        /* Jacobi: the diagonal inverse is cached on the matrix (recomputed after new values) */
        TRY(gb_mat_dinv(ctx, (gcge_gpu_mat *)g->A));
        a.dinv = g->A->dinv;
        a.dinv32 = g->A->dinv32;
    }
    if (g->conv_products) {
        /* the convergence check left A x (S2) and B x (S3) of these columns: the
         * initial residual l B w - A w, w = s x, is s (l B x - A x) without a product */
        if (g->B)
            TRY(gb_w_residual(ctx, n, wl, g->S2, g->lds, g->pos_d, g->S3, g->lds, g->pos_d, g->lam_d, g->S1,
                              g->lds));
        else
            TRY(gb_w_residual(ctx, n, wl, g->S2, g->lds, g->pos_d, g->V, g->ldv, g->unlock_d, g->lam_d, g->S1,
                              g->lds));
        a.rhs_is_residual = 1;
    } else if (g->B) {
        TRY(gb_spmm(ctx, g->B, W, g->ldv, g->S1, g->lds, wl, 1.0, g->lam_d, 0.0, NULL));
    } else {
        TRY(gb_scale_cols(ctx, n, wl, W, g->ldv, g->lam_d, g->S1, g->lds));
    }
    g->conv_products = 0;
    TRY(gb_bcg(ctx, g->A, g->S1, g->lds, W, g->ldv, &a, g->bcg_work, g->bcg_bytes));
    return 0;
fail:
    return st;
}

/* dense orthonormalisation of coefficient columns C[:, start:end) (column major,
 * nrows rows, ld ldc) against C[:, 0:start) and themselves: role of
 * GCGE_StableMultiOrthonormalizationInSubspace (src/gcge_orthogonal.c:2215-2247) */
static int orth_in_subspace(gcg_t *g, double *Cm, int ldc, int nrows, int start, int *end)
{
    gcge_gpu_ctx *ctx = g->ctx;
    int st = 0, k = *end - start;
    double *Cp = Cm + (size_t)start * ldc;
    if (k <= 0) return 0;
    if (start > 0) {
        const int passes = g->p.max_reorth_time < 1 ? 1 : g->p.max_reorth_time;
        for (int r = 0; r < passes; ++r) {
            TRY(gb_small_gemm(ctx, 'T', 'N', start, k, nrows, 1.0, Cm, ldc, Cp, ldc, 0.0, g->Gs, start));
            TRY(gb_small_gemm(ctx, 'N', 'N', nrows, k, start, -1.0, Cm, ldc, g->Gs, start, 1.0, Cp, ldc));
        }
    }
    for (int pass = 0; pass < 2 && k > 0; ++pass) {
        TRY(gb_small_gemm(ctx, 'T', 'N', k, k, nrows, 1.0, Cp, ldc, Cp, ldc, 0.0, g->Gs, k));
        TRY(gb_chol_deflate(ctx, k, g->Gs, k, g->Ts, g->kept_d, g->zero_tol, pass == 0 ? 1e-12 : 1e-14, g->chol_work));
        int kept = 0;
        CTRY(cudaMemcpyAsync(&kept, g->kept_d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CTRY(cudaStreamSynchronize(ctx->stream));
        if (kept > 0) {
            TRY(gb_small_gemm(ctx, 'N', 'N', nrows, kept, k, 1.0, Cp, ldc, g->Ts, k, 0.0, g->Ctmp, nrows));
            TRY(gb_copy_block(ctx, nrows, kept, g->Ctmp, nrows, Cp, ldc));
        }
        k = kept;
    }
    *end = start + k;
    return 0;
fail:
    return st;
}

/* GCGE_ComputeP (src/gcge_xpw.c:286-425) */
static int compute_p(gcg_t *g)
{
    gcge_gpu_ctx *ctx = g->ctx;
    int st = 0;
    const int ldc = g->dim_xpw, p_start = g->dim_x, p_ncols = g->unconv_bs, xx_nrows = g->last_dim_x;
    ph_begin(g, PH_P_ORTH);
    TRY(gb_p_coef_assemble(ctx, g->C, ldc, p_start, p_ncols, xx_nrows, g->unlock_d));
    int p_end = p_start + p_ncols;
    TRY(orth_in_subspace(g, g->C, ldc, ldc, p_start, &p_end));
    ph_end(g);
    ph_begin(g, PH_P_AXPY);
    const int p_end_tmp = p_end - g->nev;
    if (gb_lincomb_inplace_ok(ctx, ldc, p_end_tmp)) {
        /* P = V C_P written over V[:, nev:] directly (one column tile) */
        TRY(gb_lincomb(ctx, g->n, ldc, p_end_tmp, g->V, g->ldv, g->C + (size_t)g->nev * ldc, ldc, 1.0, 0.0,
                       g->V + g->nev, g->ldv, 0));
    } else {
        TRY(gb_lincomb(ctx, g->n, ldc, p_end_tmp, g->V, g->ldv, g->C + (size_t)g->nev * ldc, ldc, 1.0, 0.0, g->S1,
                       g->lds, 0));
        TRY(gb_axpby(ctx, g->n, p_end_tmp, 1.0, g->S1, g->lds, 0.0, g->V + g->nev, g->ldv));
    }
    ph_end(g);
    g->dim_xp = p_end;
    return 0;
fail:
    return st;
}

/* GCGE_CheckEvalMultiplicity (src/gcge_eigsol.c:696-718) */
static int check_multiplicity(int nev, int end, const double *eval)
{
    int t = nev;
    for (int i = nev; i < end; ++i) {
        if (fabs(fabs(eval[t] / eval[nev]) - 1) < 0.2) t += 1;
        else break;
    }
    return t;
}

static void gcg_free(gcg_t *g)
{
    void *dev[] = {g->V, g->S1, g->S2, g->S3, g->bcg_work, g->H, g->C, g->Ctmp, g->AApp, g->Gs, g->Ts,
                   g->chol_work, g->eval_d, g->eig_work, g->res_d, g->lam_d, g->dsmall, g->unlock_d, g->kept_d,
                   g->info_d, g->pos_d, g->nu_d};
    for (size_t i = 0; i < sizeof(dev) / sizeof(dev[0]); ++i)
        if (dev[i]) gb_dev_free(g->ctx, dev[i]);
    gb_orth_ws_free(&g->ows);
    free(g->eval_h);
    free(g->res_h);
    free(g->resv);
    free(g->unlock_h);
    free(g->pos_h);
    for (int i = 0; i < 128; ++i)
        if (g->tm.ev[i]) cudaEventDestroy(g->tm.ev[i]);
}

static int dmalloc(gcge_gpu_ctx *ctx, void **p, size_t bytes) { return gb_dev_alloc(ctx, p, bytes) ? 1 : 0; }

static int solve_impl(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, const gcge_gpu_params *pin,
                      double *eval, gcge_gpu_mv *evec, gcge_gpu_stats *stats);

int GCGE_GPU_Solve(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, const gcge_gpu_params *pin,
                   double *eval, gcge_gpu_mv *evec, gcge_gpu_stats *stats)
{
    if (!ctx || !A || !pin || !eval || !evec) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (pin->nev <= 0 || pin->nev > A->n || evec->ncols < pin->nev || evec->n != A->n || (B && B->n != A->n) ||
        (pin->precision && !A->v32) || pin->precision < 0 || pin->precision > 2 || pin->block_size < 0 ||
        !(pin->orth_type[0] == '\0' || ((pin->orth_type[0] == 'A' || pin->orth_type[0] == 'B') &&
                                       pin->orth_type[1] == '\0')))
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    /* precision 2: the outer products of the iteration (A W, B W, A X, B X) in
     * FP32-pair arithmetic for the duration of this solve */
    const int pair = ctx->spmm_pair;
    ctx->spmm_pair = pin->precision == 2;
    const int st = solve_impl(ctx, A, B, pin, eval, evec, stats);
    ctx->spmm_pair = pair;
    return st;
}

static int solve_impl(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, const gcge_gpu_params *pin,
                      double *eval, gcge_gpu_mv *evec, gcge_gpu_stats *stats)
{
    gcg_t G, *g = &G;
    memset(g, 0, sizeof(G));
    int st = 0;
    g->ctx = ctx;
    g->A = A;
    g->B = B;
    g->p = *pin;
    g->n = A->n;
    g->nev = pin->nev;
    g->bs = pin->block_size ? pin->block_size : pin->nev;
    g->zero_tol = pin->orth_zero_tol + DBL_EPSILON;
    g->p.w_orth_type[sizeof(g->p.w_orth_type) - 1] = '\0';
    g->orth_kind = gb_orth_kind(g->p.w_orth_type);
    g->p.orth_type[sizeof(g->p.orth_type) - 1] = '\0';
    g->amode = g->p.orth_type[0] == 'A';
    g->Om = g->amode ? A : B;
    const int nev = g->nev, n = g->n;
    /* GCGE_WORKSPACE_Setup sizes (src/gcge_workspace.c:61-73) */
    {
        int mtmp = (nev * 1.25 < nev + 8) ? (int)(nev * 1.25) : (nev + 8);
        g->max_dim_x = mtmp > nev + 3 ? mtmp : nev + 3;
    }
    g->V_size = g->max_dim_x + 2 * g->bs;
    if (g->V_size > n) {
        /* tiny problems: the basis cannot exceed the dimension */
        g->V_size = n;
        if (g->max_dim_x > n) g->max_dim_x = n;
    }
    const int vt = g->max_dim_x - nev + g->bs;
    g->S_width = nev > vt ? nev : vt;
    if (g->S_width < g->bs) g->S_width = g->bs;
    if (g->S_width < g->V_size) g->S_width = g->V_size;   /* AW and P re-combination never exceed V_size */
    g->ldv = (g->V_size + 1) & ~1;
    g->lds = (g->S_width + 1) & ~1;
    g->X = evec->d;
    g->ldx = evec->ld;
    const size_t vs = g->V_size, vs2 = vs * vs;
    for (int i = 0; i < 128; ++i)
        if (cudaEventCreate(&g->tm.ev[i]) != cudaSuccess) { st = gb_fail(ctx, GCGE_GPU_ERR_CUDA); goto fail; }
    if (dmalloc(ctx, (void **)&g->V, sizeof(double) * (size_t)n * g->ldv) || dmalloc(ctx, (void **)&g->S1, sizeof(double) * (size_t)n * g->lds) ||
        dmalloc(ctx, (void **)&g->S2, sizeof(double) * (size_t)n * g->lds) || dmalloc(ctx, (void **)&g->S3, sizeof(double) * (size_t)n * g->lds) ||
        dmalloc(ctx, (void **)&g->H, sizeof(double) * vs2) || dmalloc(ctx, (void **)&g->C, sizeof(double) * vs2) ||
        dmalloc(ctx, (void **)&g->Ctmp, sizeof(double) * vs2) || dmalloc(ctx, (void **)&g->AApp, sizeof(double) * vs2) ||
        dmalloc(ctx, (void **)&g->Gs, sizeof(double) * vs2) || dmalloc(ctx, (void **)&g->Ts, sizeof(double) * vs2) ||
        dmalloc(ctx, (void **)&g->chol_work, sizeof(double) * 2 * vs2) || dmalloc(ctx, (void **)&g->eval_d, sizeof(double) * vs) ||
        dmalloc(ctx, (void **)&g->eig_work, sizeof(double) * gb_syevx_work_doubles((int)vs)) ||
        dmalloc(ctx, (void **)&g->res_d, sizeof(double) * 3 * (nev + 8)) || dmalloc(ctx, (void **)&g->lam_d, sizeof(double) * (vs + 8)) ||
        dmalloc(ctx, (void **)&g->dsmall, sizeof(double) * 64) || dmalloc(ctx, (void **)&g->unlock_d, sizeof(int) * vs) ||
        dmalloc(ctx, (void **)&g->kept_d, sizeof(int) * 4) || dmalloc(ctx, (void **)&g->info_d, sizeof(int) * 4) ||
        dmalloc(ctx, (void **)&g->pos_d, sizeof(int) * vs) || dmalloc(ctx, (void **)&g->nu_d, sizeof(double) * vs)) {
        st = gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
        goto fail;
    }
    g->bcg_bytes = gb_bcg_work_bytes(n, g->bs, pin->precision);
    if (dmalloc(ctx, &g->bcg_work, g->bcg_bytes)) { st = gb_fail(ctx, GCGE_GPU_ERR_NOMEM); goto fail; }
    TRY(gb_orth_ws_alloc(ctx, &g->ows, n, g->V_size, g->V_size));
    g->eval_h = (double *)calloc(vs, sizeof(double));
    g->res_h = (double *)calloc(3 * (nev + 8), sizeof(double));
    g->resv = (double *)calloc(nev, sizeof(double));
    g->unlock_h = (int *)calloc(vs, sizeof(int));
    g->pos_h = (int *)calloc(vs, sizeof(int));
    if (!g->eval_h || !g->res_h || !g->resv || !g->unlock_h || !g->pos_h) { st = gb_fail(ctx, GCGE_GPU_ERR_NOMEM); goto fail; }
    CTRY(cudaMemsetAsync(g->V, 0, sizeof(double) * (size_t)n * g->ldv, ctx->stream));
    CTRY(cudaMemsetAsync(g->eval_d, 0, sizeof(double) * vs, ctx->stream));
    CTRY(cudaMemsetAsync(g->nu_d, 0, sizeof(double) * vs, ctx->stream));
    CTRY(cudaMemsetAsync(g->info_d, 0, sizeof(int), ctx->stream));
    TRY(gb_scratch(ctx, (size_t)4 * vs2 + (size_t)((n + 1023) / 1024) * 3 * (vs + 8) + (1 << 16)));
    /* GCGE_PARA_Setup (src/gcge_para.c:357-386) */
    g->num_unlock = nev;
    g->num_iter = 0;
    for (int i = 0; i < g->max_dim_x && i < (int)vs; ++i) g->unlock_h[i] = i;
    g->dim_x = nev;
    g->dim_xp = 0;
    g->dim_xpw = nev;
    g->unconv_bs = nev < g->bs ? nev : g->bs;

    cudaEvent_t e0, e1;
    CTRY(cudaEventCreate(&e0));
    CTRY(cudaEventCreate(&e1));
    const long long launches0 = ctx->launches, spmm0 = ctx->spmm_launches;
    CTRY(cudaEventRecord(e0, ctx->stream));

    /* ---- initial X (src/gcge_eigsol.c:126-212) ---- */
    ph_begin(g, PH_X_ORTH);
    {
        int have = 0;
        if (pin->given_init_evec) {
            int end = nev;
            TRY(gb_orthonormalize(ctx, n, g->X, g->ldx, 0, &end, g->Om, g->p.max_reorth_time, g->zero_tol,
                                  &g->ows));
            have = end;
        }
        for (int attempt = 0; have < nev && attempt < 16; ++attempt) {
            TRY(gb_fill_random(ctx, n, nev - have, g->X + have, g->ldx, have,
                               g->p.seed + (unsigned long long)attempt * 0x9E3779B97F4A7C15ULL));
            if (strcmp(g->p.conv_type, "O") == 0 && have == 0) {
                /* omega norm of A (src/gcge_eigsol.c:135-172) on normalised random columns */
                double *nrm = g->res_h;
                TRY(gb_col_dots(ctx, n, nev, g->X, g->ldx, g->X, g->ldx, g->res_d));
                TRY(d2h(ctx, nrm, g->res_d, sizeof(double) * nev));
                for (int i = 0; i < nev; ++i) nrm[i] = 1.0 / sqrt(nrm[i]);
                TRY(h2d(ctx, g->lam_d, nrm, sizeof(double) * nev));
                TRY(gb_scale_cols(ctx, n, nev, g->X, g->ldx, g->lam_d, g->X, g->ldx));
                TRY(gb_spmm(ctx, A, g->X, g->ldx, g->S1, g->lds, nev, 1.0, NULL, 0.0, NULL));
                TRY(gb_col_dots(ctx, n, nev, g->S1, g->lds, g->S1, g->lds, g->res_d));
                TRY(d2h(ctx, nrm, g->res_d, sizeof(double) * nev));
                double aw = 0;
                for (int i = 0; i < nev; ++i) aw += nrm[i];
                g->conv_omega_norm = sqrt(aw / nev);
            }
            if (pin->dirichlet_boundary) TRY(gb_dirichlet_zero(ctx, A, B, nev - have, g->X + have, g->ldx));
            int end = nev;
            TRY(gb_orthonormalize(ctx, n, g->X, g->ldx, have, &end, g->Om, g->p.max_reorth_time, g->zero_tol,
                                  &g->ows));
            have = end;
        }
        if (have < nev) { st = gb_fail(ctx, GCGE_GPU_ERR_BREAKDOWN); goto fail; }
    }
    ph_end(g);
    TRY(x_to_v(g));
    g->dim_xpw = g->dim_x;
    g->last_dim_x = g->dim_x;
    g->dim_xp = 0;
    ph_begin(g, PH_RR_MAT);
    TRY(rr_matrix(g));
    ph_end(g);
    ph_begin(g, PH_RR_EIGEN);
    TRY(rr_eig(g));
    ph_end(g);
    ph_begin(g, PH_X_AXPY);
    TRY(compute_x(g));
    ph_end(g);
    ph_begin(g, PH_CONV);
    TRY(check_conv(g));
    ph_end(g);
    ph_collect(g);
    TRY(x_to_v(g));
    g->dim_xp = g->dim_x;
    ph_begin(g, PH_W_LINE);
    TRY(compute_w(g));
    ph_end(g);
    g->last_dim_xpw = g->dim_xpw;
    g->dim_xpw = g->dim_xp + g->unconv_bs;
    ph_begin(g, PH_W_ORTH);
    TRY(gb_orthonormalize_kind(ctx, n, g->V, g->ldv, g->dim_x, &g->dim_xpw, g->Om, g->p.max_reorth_time,
                               g->zero_tol, &g->ows, g->orth_kind));
    ph_end(g);
    g->dim_xp = nev;
    ph_begin(g, PH_RR_MAT);
    TRY(rr_matrix(g));
    ph_end(g);
    ph_begin(g, PH_RR_EIGEN);
    TRY(rr_eig(g));
    ph_end(g);
    ph_begin(g, PH_X_AXPY);
    TRY(compute_x(g));
    ph_end(g);
    ph_begin(g, PH_CONV);
    TRY(check_conv(g));
    ph_end(g);
    ph_collect(g);

    /* ---- [X, P, W] loop (src/gcge_eigsol.c:396-528) ---- */
    for (;;) {
        while (g->num_unlock > 0 && g->num_iter < g->p.ev_max_it) {
            TRY(compute_p(g));
            TRY(x_to_v(g));
            ph_begin(g, PH_W_LINE);
            TRY(compute_w(g));
            ph_end(g);
            g->last_dim_xpw = g->dim_xpw;
            g->dim_xpw = g->dim_xp + g->unconv_bs;
            ph_begin(g, PH_W_ORTH);
            TRY(gb_orthonormalize_kind(ctx, n, g->V, g->ldv, g->dim_xp, &g->dim_xpw, g->Om, g->p.max_reorth_time,
                                       g->zero_tol, &g->ows, g->orth_kind));
            ph_end(g);
            ph_begin(g, PH_RR_MAT);
            TRY(rr_matrix(g));
            ph_end(g);
            ph_begin(g, PH_RR_EIGEN);
            TRY(rr_eig(g));
            ph_end(g);
            ph_begin(g, PH_X_AXPY);
            TRY(compute_x(g));
            ph_end(g);
            ph_begin(g, PH_CONV);
            TRY(check_conv(g));
            ph_end(g);
            ph_collect(g);
            /* CheckEvalMultiplicity on the eigenvalues check_conv brought back; ComputeX
             * only forms nev columns, so the new dim_x is first used by ComputeP */
            g->last_dim_x = g->dim_x;
            {
                const int ldm = g->dim_xpw, iu = g->max_dim_x < ldm ? g->max_dim_x : ldm;
                g->dim_x = check_multiplicity(nev, iu, g->eval_h);
            }
        }
        /* The reference only re-checks pairs that were unconverged, so a pair that
         * converged early can drift above the tolerance in later iterations. Verify
         * every pair once on exit and keep iterating on the ones above it. */
        if (g->num_unlock > 0 || g->num_iter >= g->p.ev_max_it) break;
        g->num_unlock = nev;
        for (int i = 0; i < nev; ++i) g->unlock_h[i] = i;
        g->num_iter -= 1;   /* the verification is not an iteration */
        ph_begin(g, PH_CONV);
        TRY(check_conv(g));
        ph_end(g);
        ph_collect(g);
        if (g->num_unlock == 0) break;
    }

    CTRY(cudaEventRecord(e1, ctx->stream));
    CTRY(cudaStreamSynchronize(ctx->stream));
    TRY(gb_check_device_error(ctx));
    ph_collect(g);
    memcpy(eval, g->eval_h, sizeof(double) * nev);
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        memset(stats, 0, sizeof(*stats));
        stats->num_iter = g->num_iter;
        stats->num_unlock = g->num_unlock;
        stats->max_res = g->max_res;
        stats->min_res = g->min_res;
        stats->sum_res = g->sum_res;
        stats->solve_ms = ms;
        for (int i = 0; i < PH_N; ++i) stats->phase_ms[i] = g->tm.ms[i];
        stats->kernel_launches = ctx->launches - launches0;
        stats->spmm_calls = ctx->spmm_launches - spmm0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    gcg_free(g);
    return GCGE_GPU_OK;
fail:
    cudaStreamSynchronize(ctx->stream);
    gcg_free(g);
    return st ? st : GCGE_GPU_ERR_CUDA;
}

int GCGE_GPU_SolveHost(gcge_gpu_ctx *ctx, int n, const int *A_rp, const int *A_ci, const double *A_v,
                       const int *B_rp, const int *B_ci, const double *B_v, const gcge_gpu_params *p, double *eval,
                       double *evec, gcge_gpu_stats *stats)
{
    if (!ctx || !p || !eval || !evec) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    gcge_gpu_mat *A = NULL, *B = NULL;
    gcge_gpu_mv *X = NULL;
    int st = GCGE_GPU_MatCreate(ctx, n, A_rp, A_ci, A_v, p->precision != 0, &A);
    if (!st && B_rp) st = GCGE_GPU_MatCreate(ctx, n, B_rp, B_ci, B_v, 0, &B);
    if (!st) st = GCGE_GPU_MultiVecCreate(ctx, n, p->nev, &X);
    if (!st && p->given_init_evec) st = GCGE_GPU_MultiVecUpload(X, 0, p->nev, evec);
    if (!st) st = GCGE_GPU_Solve(ctx, A, B, p, eval, X, stats);
    if (!st) st = GCGE_GPU_MultiVecDownload(X, 0, p->nev, evec);
    GCGE_GPU_MultiVecDestroy(X);
    GCGE_GPU_MatDestroy(B);
    GCGE_GPU_MatDestroy(A);
    return st;
}
