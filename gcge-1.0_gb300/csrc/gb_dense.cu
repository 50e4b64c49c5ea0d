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
__global__ void __launch_bounds__(256)
k_small_gemm(char ta, char tb, int m, int n, int k, double alpha, const double *__restrict__ A, int lda,
             const double *__restrict__ B, int ldb, double beta, double *__restrict__ C, int ldc)
{
    __shared__ double As[32][33];
    __shared__ double Bs[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    double acc[4] = {0, 0, 0, 0};
    for (int l0 = 0; l0 < k; l0 += 32) {
        for (int e = threadIdx.x; e < 1024; e += 256) {
            const int a = e & 31, b = e >> 5;  // a fastest
            // As[i][l]: op(A)(i0+i, l0+l)
            {
                const int i = a, l = b;
                const int gi = i0 + i, gl = l0 + l;
                double v = 0;
                if (gi < m && gl < k) v = (ta == 'N') ? A[gi + (long)gl * lda] : A[gl + (long)gi * lda];
                As[i][l] = v;
            }
            // Bs[l][j]: op(B)(l0+l, j0+j)
            {
                const int l = a, j = b;
                const int gl = l0 + l, gj = j0 + j;
                double v = 0;
                if (gl < k && gj < n) v = (tb == 'N') ? B[gl + (long)gj * ldb] : B[gj + (long)gl * ldb];
                Bs[l][j] = v;
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int l = 0; l < 32; ++l) {
            const double a = As[tx][l];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fma(a, Bs[l][ty + 8 * q], acc[q]);
        }
        __syncthreads();
    }
    const int i = i0 + tx;
    if (i < m) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int j = j0 + ty + 8 * q;
            if (j < n) {
                double *c = C + i + (long)j * ldc;
                *c = beta == 0.0 ? alpha * acc[q] : alpha * acc[q] + beta * *c;
            }
        }
    }
}

extern "C" int gb_small_gemm(gcge_gpu_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                             const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc)
{
    if (m <= 0 || n <= 0) return GCGE_GPU_OK;
    dim3 grid((m + 31) / 32, (n + 31) / 32);
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
               double zero_tol, double rel_tol, double *__restrict__ S, double *__restrict__ R)
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
    for (int j = 0; j < k; ++j) {
        if (tid == 0) {
            const double d = S[j + (long)j * k];
            const double g = G[j + (long)j * ldg];
            const bool ok = isfinite(d) && isfinite(g) && g > 0.0 && d > rel_tol * g && sqrt(d) > zero_tol;
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
    GB_LAUNCH(ctx, k_chol_deflate, 1, 512, 2 * k * sizeof(int), k, G, ldg, T, kept_dev, zero_tol, rel_tol, S, R);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- eigensolver
// work layout (doubles): Aw[m*m] | d[m] | e[m] | tau[m] | Zt[m*m] | lu[6*m*m] | scal[16]
extern "C" size_t gb_syevx_work_doubles(int m)
{
    return (size_t)m * m * 8 + 3 * (size_t)m + 64;
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

// one warp per wanted eigenvalue index j (il-1+warp), 32-point multisection
__global__ void __launch_bounds__(256)
k_bisect(int m, const double *__restrict__ dg, const double *__restrict__ eg, int il, int iu,
         double *__restrict__ eval, int *info)
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

__global__ void k_invit(int m, const double *__restrict__ d, const double *__restrict__ e, int nev,
                        const double *__restrict__ eval, double *__restrict__ Zt, int ldz, double *__restrict__ lu)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nev) return;
    double *dl = lu + (size_t)j * 6 * m, *dd = dl + m, *du = dd + m, *du2 = du + m, *inv = du2 + m, *ip = inv + m;
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
        dd[i] = d[i] - lam;
        dl[i] = (i < m - 1) ? e[i] : 0.0;
        du[i] = (i < m - 1) ? e[i] : 0.0;
        du2[i] = 0.0;
        ip[i] = (double)i;
    }
    for (int i = 0; i + 1 < m; ++i) {
        if (fabs(dd[i]) >= fabs(dl[i])) {
            if (dd[i] != 0.0) {
                const double f = dl[i] / dd[i];
                dl[i] = f;
                dd[i + 1] -= f * du[i];
            } else {
                dl[i] = 0.0;
            }
        } else {
            const double f = dd[i] / dl[i];
            dd[i] = dl[i];
            dl[i] = f;
            const double t = du[i];
            du[i] = dd[i + 1];
            dd[i + 1] = t - f * dd[i + 1];
            if (i + 2 < m) {
                du2[i] = du[i + 1];
                du[i + 1] = -f * du[i + 1];
            }
            ip[i] = (double)(i + 1);
        }
    }
    const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
    for (int i = 0; i < m; ++i) {
        if (fabs(dd[i]) < tiny) dd[i] = copysign(tiny, dd[i] == 0.0 ? 1.0 : dd[i]);
        inv[i] = 1.0 / dd[i];
    }
    double *z = Zt + (size_t)j * ldz;
    for (int i = 0; i < m; ++i) z[i] = start_value(j, i);
    for (int iter = 0; iter < 3; ++iter) {
        // solve L U x = z (dgttrs, no transpose)
        for (int i = 0; i + 1 < m; ++i) {
            if ((int)ip[i] == i) {
                z[i + 1] -= dl[i] * z[i];
            } else {
                const double t = z[i];
                z[i] = z[i + 1];
                z[i + 1] = t - dl[i] * z[i];
            }
        }
        z[m - 1] *= inv[m - 1];
        if (m >= 2) z[m - 2] = (z[m - 2] - du[m - 2] * z[m - 1]) * inv[m - 2];
        for (int i = m - 3; i >= 0; --i) z[i] = (z[i] - du[i] * z[i + 1] - du2[i] * z[i + 2]) * inv[i];
        double mx = 0;
        for (int i = 0; i < m; ++i) mx = fmax(mx, fabs(z[i]));
        const double s = mx > 0 ? 1.0 / mx : 1.0;
        for (int i = 0; i < m; ++i) z[i] *= s;
    }
    double nn = 0;
    for (int i = 0; i < m; ++i) nn = fma(z[i], z[i], nn);
    const double s = 1.0 / sqrt(nn);
    for (int i = 0; i < m; ++i) z[i] *= s;
}

// reorthogonalise inside clusters (gap <= 1e-3 ||T||_1, as dstein) by two
// classical Gram-Schmidt passes, then normalise. One block, vectors in order.
__global__ void __launch_bounds__(1024)
k_cluster_orth(int m, const double *__restrict__ d, const double *__restrict__ e, int nev,
               const double *__restrict__ eval, double *__restrict__ Zt, int ldz)
{
    __shared__ double coef[1024];
    __shared__ double s_tn;
    __shared__ double red[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
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
        double *zj = Zt + (size_t)j * ldz;
        const int np = j - cs;
        if (np > 0) {
            for (int pass = 0; pass < 2; ++pass) {
                for (int q = wid; q < np; q += nw) {
                    const double *zi = Zt + (size_t)(cs + q) * ldz;
                    double s = 0;
                    for (int r = lane; r < m; r += 32) s = fma(zi[r], zj[r], s);
                    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
                    if (lane == 0 && q < 1024) coef[q] = s;
                }
                __syncthreads();
                for (int r = tid; r < m; r += blockDim.x) {
                    double acc = zj[r];
                    for (int q = 0; q < np && q < 1024; ++q) acc -= coef[q] * Zt[(size_t)(cs + q) * ldz + r];
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

extern "C" int gb_syevx(gcge_gpu_ctx *ctx, int m, const double *H, int ldh, int il, int iu, double *eval,
                        double *Z, int ldz, double *work, int *info_dev)
{
    if (m <= 0 || il < 1 || iu > m || il > iu) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (m > 3000) return gb_fail(ctx, GCGE_GPU_ERR_ARG);   // dynamic shared memory of k_tridiag / k_bisect (2m doubles)
    const int nev = iu - il + 1;
    double *Aw = work, *d = Aw + (size_t)m * m, *e = d + m, *tau = e + m, *Zt = tau + m, *lu = Zt + (size_t)m * m;
    if (cudaMemsetAsync(info_dev, 0, sizeof(int), ctx->stream) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    const int tthreads = m >= 512 ? 1024 : (m >= 128 ? 512 : 256);
    GB_PROF(ctx, GB_K_EIG, 8.0 * m * m, 4.0 / 3.0 * m * (double)m * m);
    GB_LAUNCH(ctx, k_tridiag, 1, tthreads, 2 * m * sizeof(double), m, H, ldh, Aw, d, e, tau);
    const int warps_per_block = 1;     // one eigenvalue per SM: the Sturm chains use the FP64 pipe
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    GB_LAUNCH(ctx, k_bisect, (nev + warps_per_block - 1) / warps_per_block, 32 * warps_per_block,
              2 * m * sizeof(double), m, d, e, il, iu, eval, info_dev);
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    GB_LAUNCH(ctx, k_invit, (nev + 31) / 32, 32, 0, m, d, e, nev, eval, Zt, m, lu);
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    GB_LAUNCH(ctx, k_cluster_orth, 1, 1024, 0, m, d, e, nev, eval, Zt, m);
    GB_PROF(ctx, GB_K_EIG, 0.0, 0.0);
    GB_LAUNCH(ctx, k_backtransform, (nev * 32 + 255) / 256, 256, 0, m, Aw, tau, nev, Zt, m, Z, ldz);
    GB_LAUNCH(ctx, k_check_finite, 64, 256, 0, m, nev, Z, ldz, info_dev);
    return GCGE_GPU_OK;
}
