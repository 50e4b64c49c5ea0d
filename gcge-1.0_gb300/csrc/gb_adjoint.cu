// gb_adjoint.cu -- reverse-mode (adjoint) kernels of the computed eigenpairs:
// gradients of a function of eigenpairs with respect to the stored entries of A
// and B. The reference has no differentiation; these entry points extend the C
// ABI for callers that need sensitivities of A x = lambda B x.
//
// For a B-orthonormal eigenpair (lambda, x) of the symmetric pencil and a
// perturbation of one stored entry (i, j):
//   d lambda / d A_ij =  x_i x_j,          d lambda / d B_ij = -lambda x_i x_j
// (Hellmann-Feynman). For a function L(x) of a simple eigenvector with gradient
// g = dL/dx, let mu solve (A - lambda B) mu = (I - B x x^T) g with x^T B mu = 0;
// then
//   dL / d A_ij = -mu_i x_j,   dL / d B_ij = lambda mu_i x_j - (g^T x / 2) x_i x_j.
// Both are sums of products U[i, t] V[j, t] over the sparsity pattern (an SDDMM),
// which GCGE_GPU_PatternGrad evaluates; GCGE_GPU_EigvecAdjoint computes mu.
#include "gb_internal.h"

#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define GB_LAUNCH(ctx, kern, grid, block, smem, ...)                                   \
    do {                                                                               \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                 \
        (ctx)->launches++;                                                             \
        int _st = gb_check_launch(ctx);                                                \
        if (_st) return _st;                                                           \
    } while (0)

#define AD_CUDA(ctx, call)                                                             \
    do {                                                                               \
        if ((call) != cudaSuccess) return gb_fail((ctx), GCGE_GPU_ERR_CUDA);           \
    } while (0)

#define PG_THREADS 256
#define PG_LANE_MAX_R 8                 // r up to this: one lane per stored entry

// grad[e] = (acc ? grad[e] : 0) + sum_t s[t] U[i, t] V[j, t], e = (i, j) stored.
// One warp per row. Lane per stored entry (r <= PG_LANE_MAX_R): the row's scaled
// U values sit in registers and each lane gathers its V row. Otherwise the warp
// walks the row's entries and splits t over the lanes (scaled U row in shared
// memory), reducing with a fixed shuffle tree: the result does not depend on
// scheduling.
template <bool LANE_PER_ENTRY>
__global__ void __launch_bounds__(PG_THREADS)
k_pattern_grad(int n, const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ U,
               long ldu, const double *__restrict__ V, long ldv, int r, const double *__restrict__ s, int acc,
               double *__restrict__ grad)
{
    extern __shared__ double us_all[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long nw = ((long)gridDim.x * PG_THREADS) >> 5;
    for (long i = ((long)blockIdx.x * PG_THREADS + threadIdx.x) >> 5; i < n; i += nw) {
        const int beg = rp[i], end = rp[i + 1];
        if (LANE_PER_ENTRY) {
            double us[PG_LANE_MAX_R];
#pragma unroll
            for (int t = 0; t < PG_LANE_MAX_R; ++t) us[t] = t < r ? s[t] * U[i * ldu + t] : 0.0;
            for (int e = beg + lane; e < end; e += 32) {
                const double *vr = V + (long)ci[e] * ldv;
                double sum = 0.0;
#pragma unroll
                for (int t = 0; t < PG_LANE_MAX_R; ++t)
                    if (t < r) sum = fma(us[t], vr[t], sum);
                grad[e] = acc ? grad[e] + sum : sum;
            }
        } else {
            double *us = us_all + (size_t)w * r;
            for (int t = lane; t < r; t += 32) us[t] = s[t] * U[i * ldu + t];
            __syncwarp();
            for (int e = beg; e < end; ++e) {
                const double *vr = V + (long)ci[e] * ldv;
                double sum = 0.0;
                for (int t = lane; t < r; t += 32) sum = fma(us[t], vr[t], sum);
#pragma unroll
                for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
                if (lane == 0) grad[e] = acc ? grad[e] + sum : sum;
            }
            __syncwarp();
        }
    }
}

static int pg_launch(gcge_gpu_ctx *ctx, const gcge_gpu_mat *M, const double *U, long ldu, const double *V, long ldv,
                     int r, const double *s_dev, int acc, double *grad_dev)
{
    long blocks = ((long)M->n * 32 + PG_THREADS - 1) / PG_THREADS;
    const long cap = (long)ctx->num_sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    if (r <= PG_LANE_MAX_R) {
        GB_LAUNCH(ctx, k_pattern_grad<true>, (int)blocks, PG_THREADS, 0, M->n, M->rp, M->ci, U, ldu, V, ldv, r,
                  s_dev, acc, grad_dev);
    } else {
        const size_t smem = sizeof(double) * (size_t)(PG_THREADS / 32) * r;
        if (smem > 48 * 1024) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
        GB_LAUNCH(ctx, k_pattern_grad<false>, (int)blocks, PG_THREADS, smem, M->n, M->rp, M->ci, U, ldu, V, ldv, r,
                  s_dev, acc, grad_dev);
    }
    return GCGE_GPU_OK;
}

static int mv_cols_ok(const gcge_gpu_mv *m, int c0, int k)
{
    return m && c0 >= 0 && k >= 0 && c0 + k <= m->ncols;
}

extern "C" int GCGE_GPU_PatternGrad(const gcge_gpu_mat *M, const gcge_gpu_mv *U, int u0, const gcge_gpu_mv *V,
                                    int v0, int r, const double *scale, int accumulate, double *grad)
{
    if (!M || !U || !V || !scale || !grad) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = M->ctx;
    if (r < 1 || !mv_cols_ok(U, u0, r) || !mv_cols_ok(V, v0, r) || U->n != M->n || V->n != M->n ||
        (size_t)(PG_THREADS / 32) * r * sizeof(double) > 48 * 1024)
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (M->nnz == 0) return GCGE_GPU_OK;
    double *g_dev = nullptr, *s_dev = nullptr;
    int st = GCGE_GPU_OK;
    if (cudaMalloc(&g_dev, sizeof(double) * (size_t)M->nnz) != cudaSuccess ||
        cudaMalloc(&s_dev, sizeof(double) * (size_t)r) != cudaSuccess) {
        st = gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
        goto done;
    }
    if (cudaMemcpyAsync(s_dev, scale, sizeof(double) * r, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        (accumulate && cudaMemcpyAsync(g_dev, grad, sizeof(double) * (size_t)M->nnz, cudaMemcpyHostToDevice,
                                       ctx->stream) != cudaSuccess)) {
        st = gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        goto done;
    }
    st = pg_launch(ctx, M, U->d + u0, U->ld, V->d + v0, V->ld, r, s_dev, accumulate != 0, g_dev);
    if (st) goto done;
    if (cudaMemcpyAsync(grad, g_dev, sizeof(double) * (size_t)M->nnz, cudaMemcpyDeviceToHost, ctx->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        st = gb_fail(ctx, GCGE_GPU_ERR_CUDA);
done:
    cudaStreamSynchronize(ctx->stream);
    cudaFree(g_dev);
    cudaFree(s_dev);
    return st;
}

// ---------------------------------------------------------------- adjoint solve
// Work of one adjoint solve, all device resident (n-vectors contiguous, ld 1).
struct ad_work {
    double *BX;        // B X (n x m, ld m) or NULL when B = I
    double *y, *r, *p, *q, *t, *u, *w;
    double *c;         // m coefficients
    double *dot;       // one scalar
    double *h_c;       // host copy of m coefficients
};

static int ad_dot(gcge_gpu_ctx *ctx, int n, const double *x, const double *y, ad_work *W, double *out)
{
    int st = gb_col_dots(ctx, n, 1, x, 1, y, 1, W->dot);
    if (st) return st;
    AD_CUDA(ctx, cudaMemcpyAsync(out, W->dot, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    AD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!isfinite(*out)) return gb_fail(ctx, GCGE_GPU_ERR_NONFINITE);
    return GCGE_GPU_OK;
}

// dst = src - Xo (X^T Bsrc): the B-orthogonal projection onto the complement of
// X's columns (Xo = X, Bsrc = B src) or its transpose (Xo = B X, Bsrc = src)
static int ad_project(gcge_gpu_ctx *ctx, int n, int m, const double *X, long ldx, const double *Xo, long ldo,
                      const double *src, const double *Bsrc, double *dst, ad_work *W)
{
    int st = gb_gram(ctx, n, m, 1, X, ldx, Bsrc, 1, W->c, m, 0);
    if (!st && dst != src) st = gb_axpby(ctx, n, 1, 1.0, src, 1, 0.0, dst, 1);
    if (!st) st = gb_lincomb(ctx, n, m, 1, Xo, ldo, W->c, m, -1.0, 1.0, dst, 1, 0);
    return st;
}

// q = P^T (A - lambda B) P p with P = I - X X^T B (t, u, w scratch)
static int ad_apply(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, int n, int m, const double *X,
                    long ldx, double lambda, const double *p, double *q, ad_work *W)
{
    int st;
    const double *BX = W->BX ? W->BX : X;
    const long ldbx = W->BX ? m : ldx;
    // t = P p
    if (B) {
        if ((st = gb_spmm(ctx, B, p, 1, W->w, 1, 1, 1.0, nullptr, 0.0, nullptr))) return st;
        if ((st = ad_project(ctx, n, m, X, ldx, X, ldx, p, W->w, W->t, W))) return st;
    } else if ((st = ad_project(ctx, n, m, X, ldx, X, ldx, p, p, W->t, W))) {
        return st;
    }
    // u = A t - lambda B t
    if ((st = gb_spmm(ctx, A, W->t, 1, W->u, 1, 1, 1.0, nullptr, 0.0, nullptr))) return st;
    if (B) {
        if ((st = gb_spmm(ctx, B, W->t, 1, W->w, 1, 1, 1.0, nullptr, 0.0, nullptr))) return st;
        if ((st = gb_axpby(ctx, n, 1, -lambda, W->w, 1, 1.0, W->u, 1))) return st;
    } else if ((st = gb_axpby(ctx, n, 1, -lambda, W->t, 1, 1.0, W->u, 1))) {
        return st;
    }
    // q = P^T u = u - B X (X^T u)
    return ad_project(ctx, n, m, X, ldx, BX, ldbx, W->u, W->u, q, W);
}

static int ad_solve(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, int n, int m, const double *X,
                    long ldx, const double *eval, int k, const double *g, long ldg, double *mu, long ldmu,
                    double cluster_tol, double tol, int max_it, int *iters, ad_work *W)
{
    int st;
    const double lambda = eval[k];
    const double *BX = X;
    long ldbx = ldx;
    if (B) {
        if ((st = gb_spmm(ctx, B, X, ldx, W->BX, m, m, 1.0, nullptr, 0.0, nullptr))) return st;
        BX = W->BX;
        ldbx = m;
    }
    // c = X^T g; explicit components a_j = c_j / (lambda_j - lambda) outside k's cluster
    if ((st = gb_axpby(ctx, n, 1, 1.0, g, ldg, 0.0, W->r, 1))) return st;   // r = g (contiguous)
    if ((st = gb_gram(ctx, n, m, 1, X, ldx, W->r, 1, W->c, m, 0))) return st;
    AD_CUDA(ctx, cudaMemcpyAsync(W->h_c, W->c, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream));
    AD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double cscale = fmax(fabs(lambda), DBL_MIN);
    double *h_a = (double *)malloc(sizeof(double) * m);
    if (!h_a) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    for (int j = 0; j < m; ++j) {
        const double gap = eval[j] - lambda;
        h_a[j] = fabs(gap) <= cluster_tol * cscale ? 0.0 : W->h_c[j] / gap;
    }
    // b = P^T g = g - B X c  (into r), the right-hand side of the projected system
    if ((st = gb_lincomb(ctx, n, m, 1, BX, ldbx, W->c, m, -1.0, 1.0, W->r, 1, 0))) {
        free(h_a);
        return st;
    }
    // CG on P^T (A - lambda B) P y = b from y = 0
    if ((st = gb_set_zero(ctx, W->y, (size_t)n))) {
        free(h_a);
        return st;
    }
    if ((st = gb_axpby(ctx, n, 1, 1.0, W->r, 1, 0.0, W->p, 1))) {
        free(h_a);
        return st;
    }
    double rr = 0, bnorm;
    if ((st = ad_dot(ctx, n, W->r, W->r, W, &rr))) {
        free(h_a);
        return st;
    }
    bnorm = sqrt(rr);
    int it = 0;
    while (bnorm > 0 && sqrt(rr) > tol * bnorm && it < max_it) {
        double pq;
        if ((st = ad_apply(ctx, A, B, n, m, X, ldx, lambda, W->p, W->q, W))) break;
        if ((st = ad_dot(ctx, n, W->p, W->q, W, &pq))) break;
        if (!(pq > 0)) break;                               // left the SPD complement: stop
        const double alpha = rr / pq;
        if ((st = gb_axpby(ctx, n, 1, alpha, W->p, 1, 1.0, W->y, 1))) break;
        if ((st = gb_axpby(ctx, n, 1, -alpha, W->q, 1, 1.0, W->r, 1))) break;
        double rr2;
        if ((st = ad_dot(ctx, n, W->r, W->r, W, &rr2))) break;
        const double beta = rr2 / rr;
        rr = rr2;
        if ((st = gb_axpby(ctx, n, 1, 1.0, W->r, 1, beta, W->p, 1))) break;
        ++it;
    }
    if (iters) *iters = it;
    if (st) {
        free(h_a);
        return st;
    }
    // mu = P y + X a
    if (B) {
        if (!(st = gb_spmm(ctx, B, W->y, 1, W->w, 1, 1, 1.0, nullptr, 0.0, nullptr)))
            st = ad_project(ctx, n, m, X, ldx, X, ldx, W->y, W->w, W->t, W);
    } else {
        st = ad_project(ctx, n, m, X, ldx, X, ldx, W->y, W->y, W->t, W);
    }
    if (!st) {
        if (cudaMemcpyAsync(W->c, h_a, sizeof(double) * m, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
            st = gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    if (!st) st = gb_lincomb(ctx, n, m, 1, X, ldx, W->c, m, 1.0, 1.0, W->t, 1, 0);
    if (!st) st = gb_axpby(ctx, n, 1, 1.0, W->t, 1, 0.0, mu, ldmu);
    cudaStreamSynchronize(ctx->stream);
    free(h_a);
    return st;
}

extern "C" int GCGE_GPU_EigvecAdjoint(const gcge_gpu_mat *A, const gcge_gpu_mat *B, const gcge_gpu_mv *X, int m,
                                      const double *eval, int k, const gcge_gpu_mv *G, int g_col, gcge_gpu_mv *MU,
                                      int mu_col, double cluster_tol, double tol, int max_it, int *iters)
{
    if (!A || !X || !eval || !G || !MU) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = A->ctx;
    const int n = A->n;
    if (m < 1 || k < 0 || k >= m || !mv_cols_ok(X, 0, m) || !mv_cols_ok(G, g_col, 1) || !mv_cols_ok(MU, mu_col, 1) ||
        X->n != n || G->n != n || MU->n != n || (B && B->n != n) || !(cluster_tol >= 0) || !(tol > 0) ||
        max_it < 0)
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    for (int j = 0; j < m; ++j)
        if (!isfinite(eval[j])) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    ad_work W;
    memset(&W, 0, sizeof(W));
    int st = GCGE_GPU_OK;
    double *base = nullptr;
    // sub-buffers start on 256-byte boundaries
    const size_t vn = ((size_t)n + 31) & ~(size_t)31, vm = ((size_t)m + 31) & ~(size_t)31;
    const size_t nv = 7 * vn + vm + 32 + (B ? (((size_t)n * m + 31) & ~(size_t)31) : 0);
    if (cudaMalloc(&base, sizeof(double) * nv) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    W.y = base;
    W.r = W.y + vn;
    W.p = W.r + vn;
    W.q = W.p + vn;
    W.t = W.q + vn;
    W.u = W.t + vn;
    W.w = W.u + vn;
    W.c = W.w + vn;
    W.dot = W.c + vm;
    W.BX = B ? W.dot + 32 : nullptr;
    W.h_c = (double *)malloc(sizeof(double) * m);
    if (!W.h_c) {
        cudaFree(base);
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    st = ad_solve(ctx, A, B, n, m, X->d, X->ld, eval, k, G->d + g_col, G->ld, MU->d + mu_col, MU->ld, cluster_tol,
                  tol, max_it, iters, &W);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(base);
    free(W.h_c);
    return st;
}
