// gb_dense.cu -- small dense FP64 linear algebra kept resident on the GPU.
//
// The projected (Rayleigh-Ritz) matrices and the orthogonalisation Gram blocks
// are at most a few hundred wide, so these kernels are latency bound; on GB300
// the FP64 pipe also runs ~1/58 of FP32, so they are written to keep the
// dependent-operation chains short and to run independent work (eigenvalues,
// eigenvectors, columns) on separate warps or blocks.
//
//  * gb_small_gemm: column-major C = alpha op(A) op(B) + beta C.
//  * gb_chol_deflate: Cholesky of a Gram matrix with deflation of (numerically)
//    dependent columns, and the inverse of the kept triangular factor -- the
//    building block of the Cholesky-QR orthonormalisation.
//  * gb_syevx: partial symmetric eigensolver with the structure of LAPACK's
//    dsyevx for a range of indices (the routine the reference calls in
//    GCGE_Default_DenseMatEigenSolver, src/gcge_ops.c:302-316): Householder
//    tridiagonalisation, bisection on Sturm counts (32-way multisection per
//    warp), inverse iteration with reorthogonalisation inside clusters of close
//    eigenvalues, and back-transformation by the stored reflectors.
#include <cfloat>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "gb_internal.h"

#define FULL 0xffffffffu

#define GB_PROF(ctx, cls, bytes, flops) \
    do { if ((ctx)->prof) gb_prof_begin((ctx), (cls), (bytes), (flops)); } while (0)

#define GB_LAUNCH(ctx, kern, grid, block, smem, ...)                                   \
    do {                                                                               \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                 \
        (ctx)->launches++;                                                             \
        if ((ctx)->prof) gb_prof_end(ctx);                                             \
        int _st = gb_check_launch(ctx);                                                \
        if (_st) return _st;                                                           \
    } while (0)

// ---------------------------------------------------------------- small GEMM
// C = alpha op(A) op(B) + beta C for the projected matrices (m, n, k of a few hundred
// at most). FP64 on GB300 is narrow (~2 FMA per clock per SM) and a dependent FP64
// chain costs ~40 ns per step, so the work is spread thin: an 8 x 8 tile of C per
// block, 256 threads = 64 outputs x 4 slices of the inner dimension, each slice
// accumulated in two interleaved chains (k / 8 dependent steps), the slices summed
// in a fixed order in shared memory.
#define SG_T 8
__global__ void __launch_bounds__(256)
k_small_gemm(char ta, char tb, int m, int n, int k, double alpha, const double *__restrict__ A, int lda,
             const double *__restrict__ B, int ldb, double beta, double *__restrict__ C, int ldc)
{
    __shared__ double part[4][SG_T * SG_T];
    const int t = threadIdx.x, o = t & 63, sl = t >> 6;
    const int i = blockIdx.x * SG_T + (o & 7), j = blockIdx.y * SG_T + (o >> 3);
    double a0 = 0, a1 = 0;
    if (i < m && j < n) {
        const bool an = ta == 'N', bn = tb == 'N';
        int l = sl;
        for (; l + 4 < k; l += 8) {
            const double x0 = an ? A[i + (long)l * lda] : A[l + (long)i * lda];
            const double y0 = bn ? B[l + (long)j * ldb] : B[j + (long)l * ldb];
            const double x1 = an ? A[i + (long)(l + 4) * lda] : A[(l + 4) + (long)i * lda];
            const double y1 = bn ? B[(l + 4) + (long)j * ldb] : B[j + (long)(l + 4) * ldb];
            a0 = fma(x0, y0, a0);
            a1 = fma(x1, y1, a1);
        }
        if (l < k) {
            const double x0 = an ? A[i + (long)l * lda] : A[l + (long)i * lda];
            const double y0 = bn ? B[l + (long)j * ldb] : B[j + (long)l * ldb];
            a0 = fma(x0, y0, a0);
        }
    }
    part[sl][o] = a0 + a1;
    __syncthreads();
    if (sl == 0 && i < m && j < n) {
        const double acc = (part[0][o] + part[1][o]) + (part[2][o] + part[3][o]);
        double *c = C + i + (long)j * ldc;
        *c = beta == 0.0 ? alpha * acc : alpha * acc + beta * *c;
    }
}

extern "C" int gb_small_gemm(gcge_gpu_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                             const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc)
{
    if (m <= 0 || n <= 0) return GCGE_GPU_OK;
    dim3 grid((m + SG_T - 1) / SG_T, (n + SG_T - 1) / SG_T);
    GB_PROF(ctx, GB_K_DENSE, 8.0 * ((double)m * k + (double)k * n + (double)m * n), 2.0 * m * n * (double)k);
    GB_LAUNCH(ctx, k_small_gemm, grid, 256, 0, ta, tb, m, n, k > 0 ? k : 0, alpha, A, lda, B, ldb, beta, C, ldc);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- misc helpers
__global__ void k_set_zero(double *a, size_t count)
{
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x)
        a[t] = 0.0;
}
extern "C" int gb_set_zero(gcge_gpu_ctx *ctx, double *a, size_t count)
{
    if (!count) return GCGE_GPU_OK;
    size_t g = (count + 255) / 256;
    if (g > 4096) g = 4096;
    GB_LAUNCH(ctx, k_set_zero, (int)g, 256, 0, a, count);
    return GCGE_GPU_OK;
}
extern "C" int gb_copy_d(gcge_gpu_ctx *ctx, double *dst, const double *src, size_t count)
{
    if (!count) return GCGE_GPU_OK;
    if (cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    return GCGE_GPU_OK;
}
__global__ void k_set_diag(double *H, int ldh, int count, const double *vals)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        H[i + (long)i * ldh] = vals[i];
}
extern "C" int gb_set_diag_from(gcge_gpu_ctx *ctx, double *H, int ldh, int count, const double *vals)
{
    if (count <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_set_diag, (count + 255) / 256, 256, 0, H, ldh, count, vals);
    return GCGE_GPU_OK;
}
// A-orthogonal mode: the projected eigenvalues nu of -V^T B V (ascending) are
// kept in nu and turned into lambda = -1/nu (ascending as well)
__global__ void k_neg_recip(int count, double *v, double *nu)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const double x = v[i];
        nu[i] = x;
        v[i] = -1.0 / x;
    }
}
extern "C" int gb_neg_recip(gcge_gpu_ctx *ctx, int count, double *v, double *nu)
{
    if (count <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_neg_recip, (count + 255) / 256, 256, 0, count, v, nu);
    return GCGE_GPU_OK;
}
// soft locking: H[0:s, w0:m] = H[w0:m, 0:s] = 0 (the W block decoupled from the s
// locked Ritz vectors); C[:, 0:s] = e_0 .. e_(s-1); C[0:s, s:iu] = 0
__global__ void k_soft_lock(double *H, int ldh, int m, int w0, int s, double *C, int ldc, int iu)
{
    const long nh = (long)(m - w0) * s, nc = (long)m * s, nz = (long)(iu - s) * s;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nh + nc + nz; t += (long)gridDim.x * blockDim.x) {
        if (t < nh) {
            const int i = (int)(t % s), j = w0 + (int)(t / s);
            H[i + (long)j * ldh] = 0.0;
            H[j + (long)i * ldh] = 0.0;
        } else if (t < nh + nc) {
            const long u = t - nh;
            const int i = (int)(u % m), j = (int)(u / m);
            C[i + (long)j * ldc] = i == j ? 1.0 : 0.0;
        } else {
            const long u = t - nh - nc;
            const int i = (int)(u % s), j = s + (int)(u / s);
            C[i + (long)j * ldc] = 0.0;
        }
    }
}
extern "C" int gb_soft_lock(gcge_gpu_ctx *ctx, double *H, int ldh, int m, int w0, int s, double *C, int ldc, int iu)
{
    if (s <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_soft_lock, ctx->num_sms, 256, 0, H, ldh, m, w0, s, C, ldc, iu);
    return GCGE_GPU_OK;
}
__global__ void k_sym_upper(double *H, int ldh, int m)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)m * m; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % m), j = (int)(t / m);
        if (i > j) H[i + (long)j * ldh] = H[j + (long)i * ldh];
    }
}
extern "C" int gb_symmetrize_from_upper(gcge_gpu_ctx *ctx, double *H, int ldh, int m)
{
    if (m <= 1) return GCGE_GPU_OK;
    long t = (long)m * m;
    GB_LAUNCH(ctx, k_sym_upper, (int)((t + 255) / 256 > 2048 ? 2048 : (t + 255) / 256), 256, 0, H, ldh, m);
    return GCGE_GPU_OK;
}
__global__ void k_copy_block(int rows, int cols, const double *src, int lds, double *dst, int ldd)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)rows * cols; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % rows), j = (int)(t / rows);
        dst[i + (long)j * ldd] = src[i + (long)j * lds];
    }
}
extern "C" int gb_copy_block(gcge_gpu_ctx *ctx, int rows, int cols, const double *src, int lds, double *dst,
                             int ldd)
{
    if (rows <= 0 || cols <= 0) return GCGE_GPU_OK;
    long t = (long)rows * cols;
    GB_LAUNCH(ctx, k_copy_block, (int)((t + 255) / 256 > 2048 ? 2048 : (t + 255) / 256), 256, 0, rows, cols, src,
              lds, dst, ldd);
    return GCGE_GPU_OK;
}
// ComputeP coefficient assembly (src/gcge_xpw.c:325-330): zero the p_ncols columns
// starting at p_start, then copy rows xx_nrows.. of column unlock[cp] into column
// p_start+cp.
__global__ void k_p_coef(double *coef, int ldc, int p_start, int p_ncols, int xx_nrows, const int *unlock)
{
    const long total = (long)p_ncols * ldc;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int r = (int)(t % ldc), cp = (int)(t / ldc);
        double v = 0.0;
        if (r >= xx_nrows) v = coef[r + (long)unlock[cp] * ldc];
        coef[r + (long)(p_start + cp) * ldc] = v;
    }
}
extern "C" int gb_p_coef_assemble(gcge_gpu_ctx *ctx, double *coef, int ldc, int p_start, int p_ncols,
                                  int xx_nrows, const int *unlock_dev)
{
    if (p_ncols <= 0) return GCGE_GPU_OK;
    long t = (long)p_ncols * ldc;
    GB_LAUNCH(ctx, k_p_coef, (int)((t + 255) / 256), 256, 0, coef, ldc, p_start, p_ncols, xx_nrows, unlock_dev);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- Cholesky with deflation
// One block. S = G (upper used); for each column j in order: its remaining
// squared norm d = S[j,j] after removing the kept earlier columns; the column is
// dropped when d <= rel_tol * G[j,j] or sqrt(d) <= zero_tol (or not finite).
// Kept: R[j, j:] = S[j, j:] / sqrt(d), trailing update. Then U = R restricted to
// the kept rows/columns is inverted; T[K_q, p] = inv(U)[q, p] (zeros elsewhere).
__global__ void __launch_bounds__(512)
k_chol_deflate(int k, const double *__restrict__ G, int ldg, double *__restrict__ T, int *kept_out,
               double zero_tol, double rel_tol, double *__restrict__ S, double *__restrict__ R,
               double *__restrict__ min_ratio)
{
    extern __shared__ int shm[];
    int *keep = shm;            // k
    int *pos = shm + k;         // k: packed index of kept column
    __shared__ int s_drop;
    __shared__ double s_r;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (long t = tid; t < (long)k * k; t += nt) {
        const int i = (int)(t % k), j = (int)(t / k);
        S[t] = G[i + (long)j * ldg];
        R[t] = 0.0;
    }
    __syncthreads();
    double mr = 1.0;                                     // thread 0: smallest pivot / diagonal
    for (int j = 0; j < k; ++j) {
        if (tid == 0) {
            const double d = S[j + (long)j * k];
            const double g = G[j + (long)j * ldg];
            const bool ok = isfinite(d) && isfinite(g) && g > 0.0 && d > rel_tol * g && sqrt(d) > zero_tol;
            if (g > 0.0) mr = fmin(mr, d / g);
            s_drop = ok ? 0 : 1;
            s_r = ok ? sqrt(d) : 0.0;
            keep[j] = ok;
        }
        __syncthreads();
        if (!s_drop) {
            const double r = s_r, ri = 1.0 / r;
            for (int m = j + tid; m < k; m += nt) R[j + (long)m * k] = (m == j) ? r : S[j + (long)m * k] * ri;
            __syncthreads();
            const int len = k - j - 1;
            for (long t = tid; t < (long)len * len; t += nt) {
                const int a = j + 1 + (int)(t % len), b = j + 1 + (int)(t / len);
                if (a <= b) S[a + (long)b * k] -= R[j + (long)a * k] * R[j + (long)b * k];
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        int c = 0;
        for (int j = 0; j < k; ++j) { pos[j] = keep[j] ? c : -1; c += keep[j]; }
        *kept_out = c;
        if (min_ratio) *min_ratio = mr;
    }
    __syncthreads();
    // T = 0, then column p of inv(U) for each kept column j (p = pos[j]):
    // x[p] = 1/U[p,p]; x[q] = -(sum_{l=q+1..p} U[q,l] x[l]) / U[q,q], walking kept rows.
    for (long t = tid; t < (long)k * k; t += nt) T[t] = 0.0;
    __syncthreads();
    for (int jc = tid; jc < k; jc += nt) {
        if (!keep[jc]) continue;
        const int p = pos[jc];
        T[jc + (long)p * k] = 1.0 / R[jc + (long)jc * k];
        for (int q = jc - 1; q >= 0; --q) {
            if (!keep[q]) continue;
            double s0 = 0, s1 = 0;
            int l = q + 1;
            for (; l + 1 <= jc; l += 2) {
                s0 = fma(R[q + (long)l * k], T[l + (long)p * k], s0);
                s1 = fma(R[q + (long)(l + 1) * k], T[l + 1 + (long)p * k], s1);
            }
            if (l <= jc) s0 = fma(R[q + (long)l * k], T[l + (long)p * k], s0);
            T[q + (long)p * k] = -(s0 + s1) / R[q + (long)q * k];
        }
    }
}

extern "C" int gb_chol_deflate(gcge_gpu_ctx *ctx, int k, const double *G, int ldg, double *T, int *kept_dev,
                               double zero_tol, double rel_tol, double *work)
{
    if (k <= 0) return GCGE_GPU_OK;
    double *S = work, *R = work + (size_t)k * k;
    GB_LAUNCH(ctx, k_chol_deflate, 1, 512, 2 * k * sizeof(int), k, G, ldg, T, kept_dev, zero_tol, rel_tol, S, R,
              (double *)nullptr);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- eigensolver
// work layout (doubles): Aw[m*m] | d[m] | e[m] | tau[m] | Zt[m*m] | Zq[m*m] | G[m*m] | Tq[m*m] |
// cw[2*m*m] | 64 (the pivot ratio and kept count of the Cholesky-QR reorthogonalisation)
extern "C" size_t gb_syevx_work_doubles(int m)
{
    return (size_t)m * m * 7 + 3 * (size_t)m + 128;
}

// Householder reduction of the full symmetric H (lower reflectors, LAPACK dsytd2 "L").
__global__ void __launch_bounds__(1024)
k_tridiag(int m, const double *__restrict__ H, int ldh, double *__restrict__ Aw, double *__restrict__ d,
          double *__restrict__ e, double *__restrict__ tau)
{
    extern __shared__ double sm[];
    double *v = sm;          // m
    double *w = sm + m;      // m
    __shared__ double red[32];
    __shared__ double s_alpha, s_beta, s_tau, s_K;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    for (long t = tid; t < (long)m * m; t += nt) Aw[t] = H[(t % m) + (t / m) * (long)ldh];
    __syncthreads();
    for (int i = 0; i + 2 < m; ++i) {
        const int len = m - i - 1;
        double *col = Aw + (long)i * m + i + 1;           // x = Aw[i+1:m, i]
        // xn2 = ||x[1:]||^2
        double s = 0;
        for (int r = 1 + tid; r < len; r += nt) s = fma(col[r], col[r], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) red[wid] = s;
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int q = 0; q < nw; ++q) t += red[q];
            const double alpha = col[0];
            if (t == 0.0) {
                s_tau = 0.0;
                s_beta = alpha;
            } else {
                const double beta = -copysign(sqrt(alpha * alpha + t), alpha);
                s_tau = (beta - alpha) / beta;
                s_beta = beta;
                s_alpha = 1.0 / (alpha - beta);
            }
            d[i] = Aw[i + (long)i * m];
            e[i] = s_beta;
            tau[i] = s_tau;
        }
        __syncthreads();
        const double tv = s_tau;
        if (tv == 0.0) {
            for (int r = 1 + tid; r < len; r += nt) col[r] = 0.0;   // stored reflector is zero
            __syncthreads();
            continue;
        }
        const double sc = s_alpha;
        for (int r = tid; r < len; r += nt) {
            const double vr = (r == 0) ? 1.0 : col[r] * sc;
            v[r] = vr;
            if (r > 0) col[r] = vr;                            // keep v (unit lead implied)
        }
        __syncthreads();
        // p = tau * A22 v with A22 = Aw[i+1:, i+1:] held in its lower triangle:
        // warp per row r; A22[r, c] = Aw[r, c] for c <= r and Aw[c, r] for c > r.
        const double *A22 = Aw + (long)(i + 1) * m + (i + 1);
        for (int r = wid; r < len; r += nw) {
            double a0 = 0;
            for (int c = lane; c < len; c += 32) {
                const double a = (c <= r) ? A22[r + (long)c * m] : A22[c + (long)r * m];
                a0 = fma(a, v[c], a0);
            }
            for (int o = 16; o; o >>= 1) a0 += __shfl_xor_sync(FULL, a0, o);
            if (lane == 0) w[r] = tv * a0;
        }
        __syncthreads();
        // K = tau/2 * p.v
        s = 0;
        for (int r = tid; r < len; r += nt) s = fma(w[r], v[r], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) red[wid] = s;
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int q = 0; q < nw; ++q) t += red[q];
            s_K = 0.5 * tv * t;
        }
        __syncthreads();
        const double K = s_K;
        for (int r = tid; r < len; r += nt) w[r] = w[r] - K * v[r];
        __syncthreads();
        // lower triangle of A22 -= v w^T + w v^T: warp per column, lanes down the rows
        double *B22 = Aw + (long)(i + 1) * m + (i + 1);
        for (int c = wid; c < len; c += nw) {
            const double vc = v[c], wc = w[c];
            for (int r = c + lane; r < len; r += 32) B22[r + (long)c * m] -= v[r] * wc + w[r] * vc;
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (m >= 2) {
            d[m - 2] = Aw[(m - 2) + (long)(m - 2) * m];
            e[m - 2] = Aw[(m - 1) + (long)(m - 2) * m];
            tau[m - 2] = 0.0;
        }
        d[m - 1] = Aw[(m - 1) + (long)(m - 1) * m];
        e[m - 1] = 0.0;
        tau[m - 1] = 0.0;
    }
}

// The same reduction with the lower triangle packed in shared memory (column c,
// rows c..m-1, at c m - c (c - 1) / 2), for m <= TD_SMEM_MAX_M: the row-wise half
// of the matrix-vector product then reads shared memory instead of global rows
// at a stride of m doubles, and the rank-2 update stays on chip. Same operations
// in the same order as k_tridiag; the reflectors are written back to Aw (columns
// i, rows i+1..) at the end for the back-transformation.
#define TD_SMEM_MAX_M 230
static size_t td_smem_bytes(int m) { return sizeof(double) * ((size_t)m * (m + 1) / 2 + 2 * (size_t)m); }

__global__ void __launch_bounds__(1024)
k_tridiag_smem(int m, const double *__restrict__ H, int ldh, double *__restrict__ Aw, double *__restrict__ d,
               double *__restrict__ e, double *__restrict__ tau)
{
    extern __shared__ double sm[];
    double *L = sm;                                   // packed lower triangle
    double *v = sm + (size_t)m * (m + 1) / 2;         // m
    double *w = v + m;                                // m
    __shared__ double red[32];
    __shared__ double s_alpha, s_beta, s_tau, s_K;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    auto off = [m](int c) { return (long)c * m - (long)c * (c - 1) / 2; };
    for (int c = wid; c < m; c += nw)
        for (int r = c + lane; r < m; r += 32) L[off(c) + (r - c)] = H[r + (long)c * ldh];
    __syncthreads();
    for (int i = 0; i + 2 < m; ++i) {
        const int len = m - i - 1;
        double *col = L + off(i) + 1;                 // x = A[i+1:m, i]
        double s = 0;
        for (int r = 1 + tid; r < len; r += nt) s = fma(col[r], col[r], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) red[wid] = s;
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int q = 0; q < nw; ++q) t += red[q];
            const double alpha = col[0];
            if (t == 0.0) {
                s_tau = 0.0;
                s_beta = alpha;
            } else {
                const double beta = -copysign(sqrt(alpha * alpha + t), alpha);
                s_tau = (beta - alpha) / beta;
                s_beta = beta;
                s_alpha = 1.0 / (alpha - beta);
            }
            d[i] = L[off(i)];
            e[i] = s_beta;
            tau[i] = s_tau;
        }
        __syncthreads();
        const double tv = s_tau;
        if (tv == 0.0) {
            for (int r = 1 + tid; r < len; r += nt) col[r] = 0.0;
            __syncthreads();
            continue;
        }
        const double sc = s_alpha;
        for (int r = tid; r < len; r += nt) {
            const double vr = (r == 0) ? 1.0 : col[r] * sc;
            v[r] = vr;
            if (r > 0) col[r] = vr;
        }
        __syncthreads();
        // p = tau * A22 v, A22 = A[i+1:, i+1:]: warp per row r, A22[r, c] from
        // column c (c <= r) or column r (c > r) of the packed triangle
        const int b = i + 1;
        for (int r = wid; r < len; r += nw) {
            double a0 = 0;
            for (int c = lane; c < len; c += 32) {
                const double a = (c <= r) ? L[off(b + c) + (r - c)] : L[off(b + r) + (c - r)];
                a0 = fma(a, v[c], a0);
            }
            for (int o = 16; o; o >>= 1) a0 += __shfl_xor_sync(FULL, a0, o);
            if (lane == 0) w[r] = tv * a0;
        }
        __syncthreads();
        s = 0;
        for (int r = tid; r < len; r += nt) s = fma(w[r], v[r], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) red[wid] = s;
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int q = 0; q < nw; ++q) t += red[q];
            s_K = 0.5 * tv * t;
        }
        __syncthreads();
        const double K = s_K;
        for (int r = tid; r < len; r += nt) w[r] = w[r] - K * v[r];
        __syncthreads();
        for (int c = wid; c < len; c += nw) {
            const double vc = v[c], wc = w[c];
            double *Lc = L + off(b + c);
            for (int r = c + lane; r < len; r += 32) Lc[r - c] -= v[r] * wc + w[r] * vc;
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (m >= 2) {
            d[m - 2] = L[off(m - 2)];
            e[m - 2] = L[off(m - 2) + 1];
            tau[m - 2] = 0.0;
        }
        d[m - 1] = L[off(m - 1)];
        e[m - 1] = 0.0;
        tau[m - 1] = 0.0;
    }
    // reflectors (and the rest of the lower triangle) back to Aw for the back-transformation
    for (int c = wid; c < m; c += nw)
        for (int r = c + lane; r < m; r += 32) Aw[r + (long)c * m] = L[off(c) + (r - c)];
}

// 1/x by Newton-Raphson refinement of the hardware reciprocal approximation
// (rcp.approx.ftz.f64): two steps r <- r + r (1 - x r) square the relative error
// each time, leaving a few ulp. For the pivots of inverse iteration, whose
// iterate tolerates a slightly perturbed solve; an exact IEEE division costs
// several hundred cycles on this chain. Tiny or zero x take the exact division.
__device__ __forceinline__ double nr_recip(double x)
{
    if (!(fabs(x) >= DBL_MIN) || isinf(x)) return 1.0 / x;
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double t = fma(-x, r, 1.0);
    r = fma(r, t, r);
    t = fma(-x, r, 1.0);
    return fma(r, t, r);
}

// ---------------------------------------------------------------- cluster tridiagonalisation
// The same reduction as k_tridiag (dsytd2 "L": reflectors in the columns of Aw,
// d, e, tau) spread over a thread-block cluster of TC CTAs, so that the FP64 work
// of the matrix-vector product and the rank-2 update runs on TC SMs. The lower
// triangle is dealt out by columns, cyclically: column c lives in CTA c mod TC,
// rows c..m-1, packed in that CTA's shared memory. Step i:
//   A  the owner of column i forms the reflector (v, tau, beta) and publishes v;
//   B  after a cluster barrier every CTA copies v (distributed shared memory) and
//      forms its partial of p = A22 v from its own columns (row sums over the
//      columns it holds left of the row, plus the column dots below the diagonal);
//   C  after a second barrier every CTA adds the TC partials in rank order (the
//      same sum everywhere), K = tau/2 p.v, w = tau p - K v, and updates its
//      columns: A22 -= v w^T + w v^T.
// Exchange buffers alternate by step parity; barriers are the hardware cluster
// barrier (no waits on flags). All control flow is uniform over the cluster.
#define TD_THREADS 512

__device__ __forceinline__ double td_block_sum(double s, double *red)
{
    // fixed-order tree over the warps of the block (red: >= 32 doubles)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
    if (lane == 0) red[w] = s;
    __syncthreads();
    if (w == 0) {
        double t = lane < nw ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(TD_THREADS)
k_tridiag_cluster(int m, const double *__restrict__ H, int ldh, double *__restrict__ Aw, double *__restrict__ d,
                  double *__restrict__ e, double *__restrict__ tau)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int TC = (int)cl.num_blocks(), b = (int)cl.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = TD_THREADS >> 5;
    extern __shared__ double tsm[];
    __shared__ double red[33];
    __shared__ double s_tau, s_scale;
    const int ncol = b < m ? (m - 1 - b) / TC + 1 : 0;       // own columns b, b + TC, ...
    // layout: vbuf[2][m], pbuf[2][m], v[m], p[m], then the packed columns; offsets int[ncol+1] after
    double *vbuf = tsm, *pbuf = vbuf + 2 * (size_t)m, *v = pbuf + 2 * (size_t)m, *p = v + m, *A = p + m;
    long tot = 0;
    for (int l = 0; l < ncol; ++l) tot += m - (b + l * TC);
    int *off = (int *)(A + tot);
    if (tid == 0) {
        int o = 0;
        for (int l = 0; l < ncol; ++l) {
            off[l] = o;
            o += m - (b + l * TC);
        }
        off[ncol] = o;
    }
    __syncthreads();
    for (int l = 0; l < ncol; ++l) {
        const int c = b + l * TC;
        for (int r = c + tid; r < m; r += TD_THREADS) A[off[l] + (r - c)] = H[r + (long)c * ldh];
    }
    __syncthreads();
    for (int i = 0; i + 2 < m; ++i) {
        const int len = m - i - 1, par = i & 1, owner = i % TC;
        double *vb = vbuf + (size_t)par * m, *pb = pbuf + (size_t)par * m;
        // ---- A: the owner forms the reflector of column i
        if (b == owner) {
            const int l = i / TC;
            const double *col = A + off[l];               // rows i..m-1; x = rows i+1..
            double sq = 0;
            for (int r = 2 + tid; r <= len; r += TD_THREADS) sq = fma(col[r], col[r], sq);
            const double xn2 = td_block_sum(sq, red);
            if (tid == 0) {
                const double alpha = col[1];
                d[i] = col[0];
                if (xn2 == 0.0) {
                    s_tau = 0.0;
                    e[i] = alpha;
                    s_scale = 0.0;
                } else {
                    // the two quotients by Newton reciprocals (a few ulp): an IEEE
                    // division is several hundred cycles on this serial path
                    const double beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
                    s_tau = (beta - alpha) * nr_recip(beta);
                    s_scale = nr_recip(alpha - beta);
                    e[i] = beta;
                }
                tau[i] = s_tau;
            }
            __syncthreads();
            const double sc = s_scale;
            for (int r = tid; r < len; r += TD_THREADS) {
                const double vr = r == 0 ? 1.0 : col[1 + r] * sc;
                vb[r] = vr;
                if (r > 0) Aw[(long)i * m + i + 1 + r] = vr;      // stored reflector (unit lead implied)
            }
            if (tid == 0) vb[m - 1] = s_tau;                    // tau rides along in the last slot
        }
        cl.sync();
        // ---- B: copy v and tau, partial p = A22 v over the own columns
        const double *vr_own = cl.map_shared_rank(vbuf + (size_t)par * m, owner);
        for (int r = tid; r < len; r += TD_THREADS) v[r] = vr_own[r];
        if (tid == 0) s_tau = vr_own[m - 1];
        __syncthreads();
        const double tv = s_tau;
        if (tv != 0.0) {
            int l0 = (i + 1 - b + TC - 1) / TC;                  // first own column >= i + 1
            if (i + 1 <= b) l0 = 0;
            // row sums: p_b[r] = sum over own columns c <= row of A[row, c] v[c]
            for (int r = tid; r < len; r += TD_THREADS) {
                const int row = i + 1 + r;
                double a0 = 0, a1 = 0;
                int l = l0;
                for (; l + 1 < ncol && b + (l + 1) * TC <= row; l += 2) {
                    const int c0 = b + l * TC, c1 = c0 + TC;
                    a0 = fma(A[off[l] + (row - c0)], v[c0 - i - 1], a0);
                    a1 = fma(A[off[l + 1] + (row - c1)], v[c1 - i - 1], a1);
                }
                if (l < ncol && b + l * TC <= row) {
                    const int c0 = b + l * TC;
                    a0 = fma(A[off[l] + (row - c0)], v[c0 - i - 1], a0);
                }
                pb[r] = a0 + a1;
            }
            __syncthreads();
            // column dots below the diagonal: p_b[c] += sum_{row > c} A[row, c] v[row]
            for (int l = l0 + wid; l < ncol; l += nw) {
                const int c = b + l * TC;
                const double *col = A + off[l];
                double s = 0;
                for (int rr = 1 + lane; rr < m - c; rr += 32) s = fma(col[rr], v[c + rr - i - 1], s);
#pragma unroll
                for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
                if (lane == 0) pb[c - i - 1] += s;
            }
        }
        cl.sync();
        // ---- C: p = tau * sum of the partials (rank order), K, w, rank-2 update
        if (tv != 0.0) {
            for (int r = tid; r < len; r += TD_THREADS) {
                // all TC remote loads issued before the sum (rank order kept)
                double t[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) t[q] = q < TC ? cl.map_shared_rank(pbuf + (size_t)par * m, q)[r] : 0.0;
                double s = 0;
#pragma unroll
                for (int q = 0; q < 16; ++q)
                    if (q < TC) s += t[q];
                p[r] = tv * s;
            }
            __syncthreads();
            double kv = 0;
            for (int r = tid; r < len; r += TD_THREADS) kv = fma(p[r], v[r], kv);
            const double K = 0.5 * tv * td_block_sum(kv, red);
            for (int r = tid; r < len; r += TD_THREADS) p[r] -= K * v[r];     // p now holds w
            __syncthreads();
            int l0 = (i + 1 - b + TC - 1) / TC;
            if (i + 1 <= b) l0 = 0;
            for (int l = l0; l < ncol; ++l) {
                const int c = b + l * TC, cc = c - i - 1;
                const double vc = v[cc], wc = p[cc];
                double *col = A + off[l];
                for (int rr = tid; rr < m - c; rr += TD_THREADS) {
                    const int rv = cc + rr;
                    col[rr] -= v[rv] * wc + p[rv] * vc;
                }
            }
        } else if (b == owner) {
            // zero reflector: nothing to apply; the stored column below the subdiagonal is zero
            for (int r = 1 + tid; r < len; r += TD_THREADS) Aw[(long)i * m + i + 1 + r] = 0.0;
        }
        __syncthreads();
    }
    // the last two diagonal entries and the last off-diagonal
    if (m >= 2 && b == (m - 2) % TC && tid == 0) {
        const double *col = A + off[(m - 2) / TC];
        d[m - 2] = col[0];
        e[m - 2] = col[1];
        tau[m - 2] = 0.0;
    }
    if (b == (m - 1) % TC && tid == 0) {
        d[m - 1] = A[off[(m - 1) / TC]];
        e[m - 1] = 0.0;
        tau[m - 1] = 0.0;
    }
    cl.sync();                                        // no CTA leaves while others may read its buffers
}

// shared memory of k_tridiag_cluster for m and a cluster of tc CTAs (CTA 0 holds the most)
static size_t td_cluster_smem(int m, int tc)
{
    const int ncol = (m - 1) / tc + 1;
    size_t tot = 0;
    for (int l = 0; l < ncol; ++l) tot += (size_t)(m - l * tc);
    return sizeof(double) * (6 * (size_t)m + tot) + sizeof(int) * (ncol + 1) + 16;
}

// cluster size for m, 0 if the single-SM kernel is to be used
// Each of the m - 2 steps carries dependent FP64 latency (reductions, the sqrt
// and reciprocals of the reflector, two cluster barriers, the gather of the
// partial products) whatever the number of SMs, so the cluster pays only where
// a step's arithmetic on one SM (3 len^2 / 2 FMAs at ~2 FP64 FMA per clock)
// outweighs that. With the partials' remote loads issued together and Newton
// reciprocals, 16 CTAs win from m = 128 on: the dsyevx-signature call at
// m = 178 (58 wanted pairs) takes 4.69 ms against 6.45 ms with the single-SM
// reduction (8 CTAs: 4.93 ms), at m = 130 3.23 against 3.94 ms (at m = 720
// one SM would need ~60 ms of FP64 issue per reduction).
static int td_cluster_size(gcge_gpu_ctx *ctx, int m)
{
    if (m < 128) return 0;
    static int cached_m = -1, cached_tc = 0;
    if (m == cached_m) {
        if (cached_tc &&
            cudaFuncSetAttribute(k_tridiag_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)td_cluster_smem(m, cached_tc)) != cudaSuccess)
            return 0;
        return cached_tc;
    }
    cached_m = m;
    cached_tc = 0;
    static int probed = 0, allow16 = 0;
    if (!probed) {
        probed = 1;
        if (cudaFuncSetAttribute(k_tridiag_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess)
            allow16 = 1;
        cudaGetLastError();
    }
    const int want = allow16 ? 16 : 8;
    for (int tc = want; tc >= 8; tc /= 2) {
        const size_t smem = td_cluster_smem(m, tc);
        if (smem > 200 * 1024) continue;
        if (cudaFuncSetAttribute(k_tridiag_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = tc;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(tc);
        cfg.blockDim = dim3(TD_THREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_tridiag_cluster, &cfg) == cudaSuccess && nclusters > 0)
            return cached_tc = tc;
        cudaGetLastError();
    }
    (void)ctx;
    return 0;
}

static int td_cluster_launch(gcge_gpu_ctx *ctx, int tc, int m, const double *H, int ldh, double *Aw, double *d,
                             double *e, double *tau)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = tc;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(tc);
    cfg.blockDim = dim3(TD_THREADS);
    cfg.dynamicSmemBytes = td_cluster_smem(m, tc);
    cfg.stream = ctx->stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_tridiag_cluster, m, H, ldh, Aw, d, e, tau) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    ctx->launches++;
    if (ctx->prof) gb_prof_end(ctx);
    return gb_check_launch(ctx);
}

// number of eigenvalues of the tridiagonal (d, e2 = e^2) smaller than x (the
// ratio form of the Sturm sequence with the pivmin guard; its count is monotone
// in x under IEEE arithmetic, which the bisection relies on inside clusters)
__device__ __forceinline__ int sturm_count(int m, const double *d, const double *e2, double x, double pivmin)
{
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    int cnt = q < 0.0;
    for (int i = 1; i < m; ++i) {
        q = (d[i] - x) - e2[i - 1] / q;
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += q < 0.0;
    }
    return cnt;
}

// one warp per wanted eigenvalue index j (il-1+warp), 32-point multisection.
// guess (may be NULL): an estimate of each wanted eigenvalue (the previous
// Rayleigh-Ritz step's). Its first round counts at g -/+ |g| 2^-(3l+1), l = 0..15
// (lanes 0-15 below, 16-31 above); the closest points whose counts still bracket
// eigenvalue j become the interval, and the multisection goes on from there: a
// guess within relative d of the eigenvalue leaves a bracket of relative width
// ~16 d instead of the Gershgorin interval. The counts are monotone in x, so a
// wrong guess only loses that round.
__global__ void __launch_bounds__(256)
k_bisect(int m, const double *__restrict__ dg, const double *__restrict__ eg, int il, int iu,
         double *__restrict__ eval, int *info, const double *__restrict__ guess)
{
    extern __shared__ double sm[];
    double *d = sm, *e2 = sm + m;
    __shared__ double s_gl, s_gu, s_piv;
    const int tid = threadIdx.x, lane = tid & 31;
    for (int i = tid; i < m; i += blockDim.x) {
        d[i] = dg[i];
        e2[i] = (i < m - 1) ? eg[i] * eg[i] : 0.0;
    }
    __syncthreads();
    if (tid == 0) {
        double gl = DBL_MAX, gu = -DBL_MAX, emax = 0;
        for (int i = 0; i < m; ++i) {
            const double r = (i > 0 ? fabs(eg[i - 1]) : 0.0) + (i < m - 1 ? fabs(eg[i]) : 0.0);
            gl = fmin(gl, d[i] - r);
            gu = fmax(gu, d[i] + r);
            if (i < m - 1) emax = fmax(emax, e2[i]);
        }
        const double bn = fmax(fabs(gl), fabs(gu));
        const double piv = DBL_MIN * fmax(1.0, emax);
        const double fudge = 2.0 * DBL_EPSILON * bn * m + 2.0 * piv;
        s_gl = gl - fudge;
        s_gu = gu + fudge;
        s_piv = piv;
    }
    __syncthreads();
    const int j = il + (int)((blockIdx.x * blockDim.x + tid) >> 5);   // 1-based wanted index
    if (j > iu) return;                                                // warp-uniform
    double lo = s_gl, hi = s_gu;
    const double piv = s_piv;
    if (guess) {
        const double g = guess[j - il];
        if (isfinite(g) && g != 0.0) {
            const int l = lane & 15;
            const double del = ldexp(fabs(g), -(3 * l + 1));
            const double x = lane < 16 ? g - del : g + del;
            const int c = sturm_count(m, d, e2, x, piv);
            const unsigned below = __ballot_sync(FULL, lane < 16 && c < j) & 0xffffu;
            const unsigned above = __ballot_sync(FULL, lane >= 16 && c >= j) >> 16;
            if (below) {
                const double xl = __shfl_sync(FULL, x, 31 - __clz(below));
                if (xl > lo) lo = xl;
            }
            if (above) {
                const double xh = __shfl_sync(FULL, x, 16 + (31 - __clz(above)));
                if (xh < hi) hi = xh;
            }
        }
    }
    for (int it = 0; it < 80; ++it) {
        const double width = hi - lo;
        const double tolv = 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + piv;
        if (width <= tolv) break;
        const double x = lo + width * (double)(lane + 1) / 33.0;
        const int c = sturm_count(m, d, e2, x, piv);
        const unsigned ge = __ballot_sync(FULL, c >= j);
        double nlo, nhi;
        if (ge == 0u) {
            nlo = __shfl_sync(FULL, x, 31);
            nhi = hi;
        } else {
            const int f = __ffs(ge) - 1;
            nhi = __shfl_sync(FULL, x, f);
            const double xm = __shfl_sync(FULL, x, f > 0 ? f - 1 : 0);
            nlo = f > 0 ? xm : lo;
        }
        if (nlo == lo && nhi == hi) break;   // no representable progress
        lo = nlo;
        hi = nhi;
    }
    if (lane == 0) {
        const double ev = 0.5 * (lo + hi);
        eval[j - il] = ev;
        if (!isfinite(ev)) atomicExch(info, 1);
    }
}

// inverse iteration: one thread per wanted eigenvalue; LU of T - lambda I with
// partial pivoting (dgttrf layout) and three solves from a hashed start vector.
__device__ __forceinline__ double start_value(int j, int i)
{
    unsigned long long z = (unsigned long long)(j + 1) * 0x9E3779B97F4A7C15ULL ^ (unsigned long long)(i + 7) * 0xD1B54A32D192ED03ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void k_recip_probe(int n, const double *__restrict__ x, double *__restrict__ r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = nr_recip(x[i]);
}

// Internal check of nr_recip (not part of the public interface): r[i] = nr_recip(x[i])
// for n host values, on the current device.
extern "C" int gb_recip_check(int n, const double *x_host, double *r_host)
{
    if (n <= 0 || !x_host || !r_host) return GCGE_GPU_ERR_ARG;
    double *dx = nullptr, *dr = nullptr;
    int st = GCGE_GPU_OK;
    if (cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess || cudaMalloc(&dr, sizeof(double) * n) != cudaSuccess ||
        cudaMemcpy(dx, x_host, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        st = GCGE_GPU_ERR_CUDA;
    if (!st) {
        k_recip_probe<<<(n + 255) / 256, 256>>>(n, dx, dr);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(r_host, dr, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = GCGE_GPU_ERR_CUDA;
    }
    cudaFree(dx);
    cudaFree(dr);
    return st;
}

// inverse iteration: one thread per wanted eigenvalue, IV per block (one warp);
// LU of T - lambda I with partial pivoting (dgttrf layout) and three solves from
// a hashed start vector. The working arrays of the block's eigenvalues sit in
// shared memory, element i of lane l at [i * IV + l] (consecutive lanes,
// consecutive words: no bank conflicts).
__global__ void __launch_bounds__(32)
k_invit(int m, const double *__restrict__ d, const double *__restrict__ e, int nev,
        const double *__restrict__ eval, double *__restrict__ Zt, int ldz, int IV)
{
    extern __shared__ double ism[];
    const int lane = threadIdx.x;
    const int j = blockIdx.x * IV + lane;
    if (lane >= IV || j >= nev) return;
    double *dl = ism, *dd = dl + (size_t)m * IV, *du = dd + (size_t)m * IV, *du2 = du + (size_t)m * IV;
    double *inv = du2 + (size_t)m * IV, *z = inv + (size_t)m * IV;
    int *ip = (int *)(z + (size_t)m * IV);
#define IX(i) ((size_t)(i) * IV + lane)
    double tnorm = 0;
    for (int i = 0; i < m; ++i)
        tnorm = fmax(tnorm, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < m - 1 ? fabs(e[i]) : 0.0));
    // perturb a shift that repeats the previous one (dstein: separate close shifts)
    double lam = eval[j];
    const double pert = 10.0 * DBL_EPSILON * fmax(fabs(lam), tnorm * 1e-3);
    if (j > 0 && lam - eval[j - 1] < pert) {
        int k = j;
        while (k > 0 && eval[k] - eval[k - 1] < pert) --k;
        lam = eval[k] + (double)(j - k) * pert;
    }
    for (int i = 0; i < m; ++i) {
        dd[IX(i)] = d[i] - lam;
        dl[IX(i)] = (i < m - 1) ? e[i] : 0.0;
        du[IX(i)] = (i < m - 1) ? e[i] : 0.0;
        du2[IX(i)] = 0.0;
        ip[IX(i)] = i;
    }
    for (int i = 0; i + 1 < m; ++i) {
        const double di = dd[IX(i)], li = dl[IX(i)];
        if (fabs(di) >= fabs(li)) {
            if (di != 0.0) {
                const double f = li * nr_recip(di);
                dl[IX(i)] = f;
                dd[IX(i + 1)] -= f * du[IX(i)];
            } else {
                dl[IX(i)] = 0.0;
            }
        } else {
            const double f = di * nr_recip(li);
            dd[IX(i)] = li;
            dl[IX(i)] = f;
            const double t = du[IX(i)];
            const double dn = dd[IX(i + 1)];
            du[IX(i)] = dn;
            dd[IX(i + 1)] = t - f * dn;
            if (i + 2 < m) {
                du2[IX(i)] = du[IX(i + 1)];
                du[IX(i + 1)] = -f * du[IX(i + 1)];
            }
            ip[IX(i)] = i + 1;
        }
    }
    const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
    for (int i = 0; i < m; ++i) {
        double di = dd[IX(i)];
        if (fabs(di) < tiny) di = copysign(tiny, di == 0.0 ? 1.0 : di);
        dd[IX(i)] = di;
        inv[IX(i)] = nr_recip(di);
    }
    for (int i = 0; i < m; ++i) z[IX(i)] = start_value(j, i);
    for (int iter = 0; iter < 3; ++iter) {
        // solve L U x = z (dgttrs, no transpose)
        for (int i = 0; i + 1 < m; ++i) {
            if (ip[IX(i)] == i) {
                z[IX(i + 1)] -= dl[IX(i)] * z[IX(i)];
            } else {
                const double t = z[IX(i)];
                z[IX(i)] = z[IX(i + 1)];
                z[IX(i + 1)] = t - dl[IX(i)] * z[IX(i)];
            }
        }
        z[IX(m - 1)] *= inv[IX(m - 1)];
        if (m >= 2) z[IX(m - 2)] = (z[IX(m - 2)] - du[IX(m - 2)] * z[IX(m - 1)]) * inv[IX(m - 2)];
        for (int i = m - 3; i >= 0; --i)
            z[IX(i)] = (z[IX(i)] - du[IX(i)] * z[IX(i + 1)] - du2[IX(i)] * z[IX(i + 2)]) * inv[IX(i)];
        double mx = 0;
        for (int i = 0; i < m; ++i) mx = fmax(mx, fabs(z[IX(i)]));
        const double sc = mx > 0 ? 1.0 / mx : 1.0;
        for (int i = 0; i < m; ++i) z[IX(i)] *= sc;
    }
    double nn = 0;
    for (int i = 0; i < m; ++i) nn = fma(z[IX(i)], z[IX(i)], nn);
    const double sc = 1.0 / sqrt(nn);
    double *zo = Zt + (size_t)j * ldz;
    for (int i = 0; i < m; ++i) zo[i] = z[IX(i)] * sc;
#undef IX
}

// reorthogonalise inside clusters (gap <= 1e-3 ||T||_1, as dstein) by two
// classical Gram-Schmidt passes, then normalise. One block, vectors in order;
// with SMEM the nev vectors are worked on in shared memory (m * nev doubles).
template <bool SMEM>
__global__ void __launch_bounds__(1024)
k_cluster_orth(int m, const double *__restrict__ d, const double *__restrict__ e, int nev,
               const double *__restrict__ eval, double *__restrict__ Zg, int ldz)
{
    extern __shared__ double zsm[];
    __shared__ double coef[1024];
    __shared__ double s_tn;
    __shared__ double red[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    double *Zt = Zg;
    long ld = ldz;
    if (SMEM) {
        for (long t = tid; t < (long)m * nev; t += blockDim.x) zsm[t] = Zg[(t / m) * ldz + t % m];
        Zt = zsm;
        ld = m;
    }
    if (tid == 0) {
        double t = 0;
        for (int i = 0; i < m; ++i)
            t = fmax(t, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < m - 1 ? fabs(e[i]) : 0.0));
        s_tn = t;
    }
    __syncthreads();
    const double ortol = 1e-3 * s_tn;
    int cs = 0;
    for (int j = 0; j < nev; ++j) {
        if (j > 0 && eval[j] - eval[j - 1] > ortol) cs = j;
        double *zj = Zt + (size_t)j * ld;
        const int np = j - cs;
        if (np > 0) {
            for (int pass = 0; pass < 2; ++pass) {
                for (int q = wid; q < np; q += nw) {
                    const double *zi = Zt + (size_t)(cs + q) * ld;
                    double s = 0;
                    for (int r = lane; r < m; r += 32) s = fma(zi[r], zj[r], s);
                    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
                    if (lane == 0 && q < 1024) coef[q] = s;
                }
                __syncthreads();
                for (int r = tid; r < m; r += blockDim.x) {
                    double acc = zj[r];
                    for (int q = 0; q < np && q < 1024; ++q) acc -= coef[q] * Zt[(size_t)(cs + q) * ld + r];
                    zj[r] = acc;
                }
                __syncthreads();
            }
        }
        double s = 0;
        for (int r = tid; r < m; r += blockDim.x) s = fma(zj[r], zj[r], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) red[wid] = s;
        __syncthreads();
        if (tid == 0) {
            double t = 0;
            for (int q = 0; q < nw; ++q) t += red[q];
            red[0] = t > 0 ? 1.0 / sqrt(t) : 1.0;
        }
        __syncthreads();
        const double inv = red[0];
        for (int r = tid; r < m; r += blockDim.x) zj[r] *= inv;
        __syncthreads();
    }
    if (SMEM)
        for (long t = tid; t < (long)m * nev; t += blockDim.x) Zg[(t / m) * ldz + t % m] = zsm[t];
}

// Z = Q Zt with Q = H_0 H_1 ... H_{m-3}; one warp per column, reflectors in reverse.
__global__ void __launch_bounds__(256)
k_backtransform(int m, const double *__restrict__ Aw, const double *__restrict__ tau, int nev,
                const double *__restrict__ Zt, int ldzt, double *__restrict__ Z, int ldz)
{
    const int lane = threadIdx.x & 31;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nev) return;
    double *z = Z + (size_t)c * ldz;
    const double *zt = Zt + (size_t)c * ldzt;
    for (int r = lane; r < m; r += 32) z[r] = zt[r];
    __syncwarp();
    for (int i = m - 3; i >= 0; --i) {
        const double t = tau[i];
        if (t == 0.0) continue;
        const double *v = Aw + (size_t)i * m;   // v[i+1] = 1, v[i+2:] stored
        double s = 0;
        for (int r = i + 1 + lane; r < m; r += 32) s = fma(r == i + 1 ? 1.0 : v[r], z[r], s);
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        const double f = t * s;
        for (int r = i + 1 + lane; r < m; r += 32) z[r] -= f * (r == i + 1 ? 1.0 : v[r]);
        __syncwarp();
    }
}

__global__ void k_check_finite(int m, int nev, const double *Z, int ldz, int *info)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)m * nev; t += (long)gridDim.x * blockDim.x)
        if (!isfinite(Z[(t % m) + (t / m) * (long)ldz])) atomicExch(info, 2);
}

// Reorthogonalisation of many inverse-iteration vectors by Cholesky-QR.
// k_cluster_orth orthogonalises each vector against the earlier members of its
// cluster (eigenvalues closer than 1e-3 ||T||, dstein's criterion) by modified
// Gram-Schmidt in one thread block; when ||T|| is large against the wanted
// eigenvalues (a graph pencil: projected spectrum to ~2e3, wanted ones below 1)
// every wanted vector falls in one cluster, and that block does O(nev^2 m) FP64
// work alone. Gram-Schmidt over all vectors in index order is the Q factor of
// Z = Q R, which Cholesky-QR computes with parallel small GEMMs: G = Z^T Z,
// R^T R = G, Z <- Z R^-1. Inverse-iteration vectors are nearly orthonormal, so
// one pass leaves them orthonormal to rounding when every pivot keeps at least
// half of its column's norm squared (condition number of Z below ~1.5); a second
// pass repairs the first one's rounding otherwise. Vectors of well-separated
// eigenvalues are already orthogonal to O(eps ||T|| / gap), so the mixing
// outside the clusters is of that order. A pivot below 1e-10 of its column's
// norm (nearly dependent vectors) keeps the vectors as they were and the caller
// falls back to k_cluster_orth. (m = 720, nev = 208, one GB300: 33 ms per
// dsyevx-signature call against 44.5 ms with k_cluster_orth, both passes run.)
#define CQ_MIN_NEV 96
static int cholqr_reorth(gcge_gpu_ctx *ctx, int m, int nev, double *Zt, double *ext, int *done)
{
    double *Zq = ext, *G = Zq + (size_t)m * m, *Tq = G + (size_t)m * m, *cw = Tq + (size_t)m * m;
    double *ratio_dev = cw + 2 * (size_t)m * m;
    int *kept_dev = (int *)(ratio_dev + 8);
    *done = 0;
    for (int pass = 0; pass < 2; ++pass) {
        double *src = pass == 0 ? Zt : Zq, *dst = pass == 0 ? Zq : Zt;
        int st = gb_small_gemm(ctx, 'T', 'N', nev, nev, m, 1.0, src, m, src, m, 0.0, G, nev);
        if (st) return st;
        GB_LAUNCH(ctx, k_chol_deflate, 1, 512, 2 * nev * sizeof(int), nev, G, nev, Tq, kept_dev, 0.0, 1e-10, cw,
                  cw + (size_t)nev * nev, ratio_dev);
        struct { int kept; int pad; double ratio; } h = {0, 0, 0.0};
        if (cudaMemcpyAsync(&h.kept, kept_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaMemcpyAsync(&h.ratio, ratio_dev, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess)
            return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        if (h.kept != nev) {
            // nearly dependent vectors: leave them (the second pass' input is copied back)
            if (pass == 1 && (st = gb_copy_block(ctx, m, nev, Zq, m, Zt, m))) return st;
            return GCGE_GPU_OK;
        }
        if ((st = gb_small_gemm(ctx, 'N', 'N', m, nev, nev, 1.0, src, m, Tq, nev, 0.0, dst, m))) return st;
        if (pass == 0 && h.ratio >= 0.5) {
            if ((st = gb_copy_block(ctx, m, nev, Zq, m, Zt, m))) return st;
            break;
        }
    }
    *done = 1;
    return GCGE_GPU_OK;
}

extern "C" int gb_syevx_guess(gcge_gpu_ctx *ctx, int m, const double *H, int ldh, int il, int iu, double *eval,
                              double *Z, int ldz, double *work, int *info_dev, const double *guess);
extern "C" int gb_syevx(gcge_gpu_ctx *ctx, int m, const double *H, int ldh, int il, int iu, double *eval,
                        double *Z, int ldz, double *work, int *info_dev)
{
    return gb_syevx_guess(ctx, m, H, ldh, il, iu, eval, Z, ldz, work, info_dev, nullptr);
}

extern "C" int gb_syevx_guess(gcge_gpu_ctx *ctx, int m, const double *H, int ldh, int il, int iu, double *eval,
                              double *Z, int ldz, double *work, int *info_dev, const double *guess)
{
    if (m <= 0 || il < 1 || iu > m || il > iu) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (m > 3000) return gb_fail(ctx, GCGE_GPU_ERR_ARG);   // dynamic shared memory of k_tridiag / k_bisect (2m doubles)
    const int nev = iu - il + 1;
    double *Aw = work, *d = Aw + (size_t)m * m, *e = d + m, *tau = e + m, *Zt = tau + m;
    if (cudaMemsetAsync(info_dev, 0, sizeof(int), ctx->stream) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    const int tthreads = m >= 512 ? 1024 : (m >= 128 ? 512 : 256);
    GB_PROF(ctx, GB_K_EIG, 8.0 * m * m, 4.0 / 3.0 * m * (double)m * m);
    const int tc = td_cluster_size(ctx, m);
    if (tc) {
        int st = td_cluster_launch(ctx, tc, m, H, ldh, Aw, d, e, tau);
        if (st) return st;
    } else {
        static bool td_attr = false;
        if (!td_attr) {
            if (cudaFuncSetAttribute(k_tridiag_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)td_smem_bytes(TD_SMEM_MAX_M)) != cudaSuccess)
                return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
            td_attr = true;
        }
        if (m <= TD_SMEM_MAX_M)
            GB_LAUNCH(ctx, k_tridiag_smem, 1, tthreads, td_smem_bytes(m), m, H, ldh, Aw, d, e, tau);
        else
            GB_LAUNCH(ctx, k_tridiag, 1, tthreads, 2 * m * sizeof(double), m, H, ldh, Aw, d, e, tau);
    }
    const int warps_per_block = 1;     // one eigenvalue per SM: the Sturm chains use the FP64 pipe
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    GB_LAUNCH(ctx, k_bisect, (nev + warps_per_block - 1) / warps_per_block, 32 * warps_per_block,
              2 * m * sizeof(double), m, d, e, il, iu, eval, info_dev, guess);
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    // inverse iteration: one eigenvalue per one-warp block, so that the chains spread
    // over the SMs (the FP64 pipe of an SM is narrow: chains sharing one SM queue
    // on it); working arrays in shared memory
    const size_t per_eig = (size_t)m * (6 * sizeof(double) + sizeof(int));
    const int IV = 1;
    const size_t ismem = per_eig * IV;
    // the 48 KB default covers static + dynamic shared memory together: both kernels
    // are opened once to the most they can ask for (k_invit <= 156 KB at m = 3000,
    // k_cluster_orth<true> <= 160 KB + its 8.3 KB static)
    static bool attrs = false;
    if (!attrs) {
        if (cudaFuncSetAttribute(k_invit, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024) != cudaSuccess ||
            cudaFuncSetAttribute(k_cluster_orth<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024) !=
                cudaSuccess)
            return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        attrs = true;
    }
    GB_LAUNCH(ctx, k_invit, (nev + IV - 1) / IV, 32, ismem, m, d, e, nev, eval, Zt, m, IV);
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    int reorth_done = 0;
    if (nev >= CQ_MIN_NEV) {
        const int st = cholqr_reorth(ctx, m, nev, Zt, Zt + (size_t)m * m, &reorth_done);
        if (st) return st;
    }
    const size_t osmem = sizeof(double) * (size_t)m * nev;
    if (reorth_done) {
        // the vectors are orthonormal: Cholesky-QR over all of them
    } else if (osmem <= 160 * 1024) {
        GB_LAUNCH(ctx, k_cluster_orth<true>, 1, 1024, osmem, m, d, e, nev, eval, Zt, m);
    } else {
        GB_LAUNCH(ctx, k_cluster_orth<false>, 1, 1024, 0, m, d, e, nev, eval, Zt, m);
    }
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    GB_LAUNCH(ctx, k_backtransform, (nev * 32 + 255) / 256, 256, 0, m, Aw, tau, nev, Zt, m, Z, ldz);
    GB_LAUNCH(ctx, k_check_finite, 64, 256, 0, m, nev, Z, ldz, info_dev);
    return GCGE_GPU_OK;
}
