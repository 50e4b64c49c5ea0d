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

// ---------------------------------------------------------------- single-vector kernels
// The adjoint CG works on one n-vector at a time; these kernels are sized for
// that (the block kernels of the solver are not).
#define AV_THREADS 256
#define AV_BLOCKS_PER_SM 4

static int av_grid(gcge_gpu_ctx *ctx, long work)
{
    long g = (work + AV_THREADS - 1) / AV_THREADS, cap = (long)ctx->num_sms * AV_BLOCKS_PER_SM;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// y = a x + b y (b == 0: y = a x, y not read)
__global__ void k_av_axpby(long n, double a, const double *__restrict__ x, double b, double *__restrict__ y)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = b == 0.0 ? a * x[i] : fma(a, x[i], b * y[i]);
}

// part[block] = sum over the block's grid-stride slice of x_i y_i (fixed order)
__global__ void __launch_bounds__(AV_THREADS)
k_av_dot_part(long n, const double *__restrict__ x, const double *__restrict__ y, double *__restrict__ part)
{
    __shared__ double red[AV_THREADS / 32];
    double s = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        s = fma(x[i], y[i], s);
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < AV_THREADS / 32; ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

// out[0] = sum of nparts partials (one warp, fixed order)
__global__ void k_av_sum(int nparts, const double *__restrict__ part, double *__restrict__ out)
{
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += 32) s += part[i];
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = s;
}

// part[block][j] = sum over the block's rows of X[r, j] v[r], j < m <= 64: a warp
// per row, lanes over the columns (a row of X is contiguous)
__global__ void __launch_bounds__(AV_THREADS)
k_av_xtv_part(long n, int m, const double *__restrict__ X, long ldx, const double *__restrict__ v,
              double *__restrict__ part)
{
    __shared__ double red[AV_THREADS / 32][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double s0 = 0.0, s1 = 0.0;
    const long nw = ((long)gridDim.x * AV_THREADS) >> 5;
    for (long r = ((long)blockIdx.x * AV_THREADS + threadIdx.x) >> 5; r < n; r += nw) {
        const double vr = v[r];
        const double *xr = X + r * ldx;
        if (lane < m) s0 = fma(xr[lane], vr, s0);
        if (lane + 32 < m) s1 = fma(xr[lane + 32], vr, s1);
    }
    red[w][lane] = s0;
    red[w][lane + 32] = s1;
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += AV_THREADS) {
        double t = 0.0;
        for (int q = 0; q < AV_THREADS / 32; ++q) t += red[q][j];
        part[(long)blockIdx.x * m + j] = t;
    }
}

// c[j] = sum of the partials of column j (thread per column, fixed order)
__global__ void k_av_xtv_sum(int nparts, int m, const double *__restrict__ part, double *__restrict__ c)
{
    const int j = threadIdx.x;
    if (j >= m) return;
    double t = 0.0;
    for (int b = 0; b < nparts; ++b) t += part[(long)b * m + j];
    c[j] = t;
}

// y = v - X c (thread per row, c in shared memory), m <= 64
__global__ void __launch_bounds__(AV_THREADS)
k_av_v_minus_xc(long n, int m, const double *__restrict__ X, long ldx, const double *__restrict__ c,
                const double *__restrict__ v, double *__restrict__ y)
{
    __shared__ double cs[64];
    if (threadIdx.x < m) cs[threadIdx.x] = c[threadIdx.x];
    __syncthreads();
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
        const double *xr = X + r * ldx;
        double s = 0.0;
        for (int j = 0; j < m; ++j) s = fma(xr[j], cs[j], s);
        y[r] = v[r] - s;
    }
}

// ---------------------------------------------------------------- adjoint solve
// Work of one adjoint solve, all device resident (n-vectors contiguous, ld 1).
struct ad_work {
    double *BX;        // B X (n x m, ld m) or NULL when B = I
    double *y, *r, *p, *q, *t, *u, *w;
    double *c;         // m coefficients
    double *dot;       // one scalar
    double *part;      // block partials (grid x max(m, 1))
    double *h_c;       // host copy of m coefficients
};

#define AD_SKINNY_M 64                  // widest X handled by the single-vector kernels

static int ad_axpby(gcge_gpu_ctx *ctx, int n, double a, const double *x, double b, double *y)
{
    GB_LAUNCH(ctx, k_av_axpby, av_grid(ctx, n), AV_THREADS, 0, (long)n, a, x, b, y);
    return GCGE_GPU_OK;
}

static int ad_dot(gcge_gpu_ctx *ctx, int n, const double *x, const double *y, ad_work *W, double *out)
{
    const int g = av_grid(ctx, n);
    GB_LAUNCH(ctx, k_av_dot_part, g, AV_THREADS, 0, (long)n, x, y, W->part);
    GB_LAUNCH(ctx, k_av_sum, 1, 32, 0, g, W->part, W->dot);
    AD_CUDA(ctx, cudaMemcpyAsync(out, W->dot, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    AD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!isfinite(*out)) return gb_fail(ctx, GCGE_GPU_ERR_NONFINITE);
    return GCGE_GPU_OK;
}

// c = X^T v (m coefficients, device)
static int ad_xtv(gcge_gpu_ctx *ctx, int n, int m, const double *X, long ldx, const double *v, double *c, ad_work *W)
{
    if (m > AD_SKINNY_M) return gb_gram(ctx, n, m, 1, X, ldx, v, 1, c, m, 0);
    const int g = av_grid(ctx, (long)n * 32);
    GB_LAUNCH(ctx, k_av_xtv_part, g, AV_THREADS, 0, (long)n, m, X, ldx, v, W->part);
    GB_LAUNCH(ctx, k_av_xtv_sum, 1, 64, 0, g, m, W->part, c);
    return GCGE_GPU_OK;
}

// y = v - X c (y may be v)
static int ad_v_minus_xc(gcge_gpu_ctx *ctx, int n, int m, const double *X, long ldx, const double *c,
                         const double *v, double *y)
{
    if (m > AD_SKINNY_M) {
        int st = y != v ? ad_axpby(ctx, n, 1.0, v, 0.0, y) : GCGE_GPU_OK;
        return st ? st : gb_lincomb(ctx, n, m, 1, X, ldx, c, m, -1.0, 1.0, y, 1, 0);
    }
    GB_LAUNCH(ctx, k_av_v_minus_xc, av_grid(ctx, n), AV_THREADS, 0, (long)n, m, X, ldx, c, v, y);
    return GCGE_GPU_OK;
}

// dst = src - Xo (X^T Bsrc): the B-orthogonal projection onto the complement of
// X's columns (Xo = X, Bsrc = B src) or its transpose (Xo = B X, Bsrc = src)
static int ad_project(gcge_gpu_ctx *ctx, int n, int m, const double *X, long ldx, const double *Xo, long ldo,
                      const double *src, const double *Bsrc, double *dst, ad_work *W)
{
    int st = ad_xtv(ctx, n, m, X, ldx, Bsrc, W->c, W);
    return st ? st : ad_v_minus_xc(ctx, n, m, Xo, ldo, W->c, src, dst);
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
        if ((st = ad_axpby(ctx, n, -lambda, W->w, 1.0, W->u))) return st;
    } else if ((st = ad_axpby(ctx, n, -lambda, W->t, 1.0, W->u))) {
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
    if ((st = ad_xtv(ctx, n, m, X, ldx, W->r, W->c, W))) return st;
    AD_CUDA(ctx, cudaMemcpyAsync(W->h_c, W->c, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream));
    AD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double cscale = fmax(fabs(lambda), DBL_MIN);
    double *h_a = (double *)malloc(sizeof(double) * m);
    if (!h_a) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    for (int j = 0; j < m; ++j) {
        const double gap = eval[j] - lambda;
        h_a[j] = fabs(gap) <= cluster_tol * cscale ? 0.0 : -W->h_c[j] / gap;   // negated: v - X c form
    }
    double rr = 0, bnorm = 0;
    int it = 0;
    // b = P^T g = g - B X c (into r), the right-hand side of the projected system;
    // CG on P^T (A - lambda B) P y = b from y = 0
    st = ad_v_minus_xc(ctx, n, m, BX, ldbx, W->c, W->r, W->r);
    if (!st) st = gb_set_zero(ctx, W->y, (size_t)n);
    if (!st) st = ad_axpby(ctx, n, 1.0, W->r, 0.0, W->p);
    if (!st) st = ad_dot(ctx, n, W->r, W->r, W, &rr);
    bnorm = sqrt(rr);
    while (!st && bnorm > 0 && sqrt(rr) > tol * bnorm && it < max_it) {
        double pq;
        if ((st = ad_apply(ctx, A, B, n, m, X, ldx, lambda, W->p, W->q, W))) break;
        if ((st = ad_dot(ctx, n, W->p, W->q, W, &pq))) break;
        if (!(pq > 0)) break;                               // left the SPD complement: stop
        const double alpha = rr / pq;
        if ((st = ad_axpby(ctx, n, alpha, W->p, 1.0, W->y))) break;
        if ((st = ad_axpby(ctx, n, -alpha, W->q, 1.0, W->r))) break;
        double rr2;
        if ((st = ad_dot(ctx, n, W->r, W->r, W, &rr2))) break;
        const double beta = rr2 / rr;
        rr = rr2;
        if ((st = ad_axpby(ctx, n, 1.0, W->r, beta, W->p))) break;
        ++it;
    }
    if (iters) *iters = it;
    // mu = P y + X a
    if (!st) {
        if (B) {
            if (!(st = gb_spmm(ctx, B, W->y, 1, W->w, 1, 1, 1.0, nullptr, 0.0, nullptr)))
                st = ad_project(ctx, n, m, X, ldx, X, ldx, W->y, W->w, W->t, W);
        } else {
            st = ad_project(ctx, n, m, X, ldx, X, ldx, W->y, W->y, W->t, W);
        }
    }
    if (!st && cudaMemcpyAsync(W->c, h_a, sizeof(double) * m, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
        st = gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    if (!st) st = ad_v_minus_xc(ctx, n, m, X, ldx, W->c, W->t, W->t);
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
    const size_t np = (((size_t)ctx->num_sms * AV_BLOCKS_PER_SM * (size_t)(m > 1 ? m : 1)) + 31) & ~(size_t)31;
    const size_t nv = 7 * vn + vm + 32 + np + (B ? (((size_t)n * m + 31) & ~(size_t)31) : 0);
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
    W.part = W.dot + 32;
    W.BX = B ? W.part + np : nullptr;
    W.h_c = (double *)malloc(sizeof(double) * m);
    if (!W.h_c) {
        cudaFree(base);
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    // the projections are n x m by one column: FP64-pipe Gram and combination
    // kernels (no tensor-core set-up per call)
    const int tc = ctx->tc;
    ctx->tc = 0;
    st = ad_solve(ctx, A, B, n, m, X->d, X->ld, eval, k, G->d + g_col, G->ld, MU->d + mu_col, MU->ld, cluster_tol,
                  tol, max_it, iters, &W);
    ctx->tc = tc;
    cudaStreamSynchronize(ctx->stream);
    cudaFree(base);
    free(W.h_c);
    return st;
}
