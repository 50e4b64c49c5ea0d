// gb_bcg.cu -- block conjugate gradients on GB300, GCGE_BCG semantics
// (src/gcge_cg.c:137-302) with all control state on the device.
//
// Per-column scalars rho1, rho2, ptw, err and the active-column count live in
// device memory; every kernel reads the count and leaves columns at or beyond it
// untouched, so the loop runs cg_max_it-1 rounds without a host round trip and
// a round with no active column costs only its launches.
//
// The active set follows the reference exactly: after each round the count of
// columns whose residual ratio ||r_k||/||r_0|| is still >= cg_rate is taken
// over all columns, and the next round updates the first `count` columns
// (src/gcge_cg.c:286-294 writes unlock[idx] = idx at position idx, and the
// update loops walk unlock[0 .. num_unlock)).
//
// precision 0: FP64 vectors and values. precision 1: the residual of the initial
// guess is formed in FP64, then CG runs on the correction with FP32 vectors and
// the FP32 copy of the matrix values; products are formed in FP32 and summed in
// FP32 over runs of 8 rows, then accumulated in FP64 (FP64-reduced dot products);
// the correction is added to the FP64 solution at the end.
#include <cuda_runtime.h>

#include "gb_internal.h"

#define RED_ROWS 128

extern "C" int gb_axpy32(gcge_gpu_ctx *ctx, int n, int k, float a, const float *X, float *Y, long ld);

static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

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

struct bcg_state {
    double *rho1, *rho2, *err, *ptw, *part, *alpha, *beta, *sums;
    int *nact;
};

// warp-per-row loop over an n x k block: lanes walk the columns of one row
#define ROWS_BY_WARP(n, r)                                                             \
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (n);         \
         r += ((long)gridDim.x * blockDim.x) >> 5)

// p = r + beta p on active columns (beta = 0 on the first round: p = r);
// beta[c] = rho2[c] / rho1[c] was formed once per column by k_finalize
template <typename T>
__global__ void k_pupdate(int n, int k, const T *__restrict__ R, T *__restrict__ P, long ld,
                          const double *__restrict__ beta, const int *__restrict__ nact, int first,
                          const T *__restrict__ dinv)
{
    const int ka = min(*nact, k);
    if (ka <= 0) return;
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    {
        const T *rr = R + r * ld;
        T *pr = P + r * ld;
        const T dr = dinv ? dinv[r] : (T)1;                // z = D^-1 r (Jacobi) or r
        for (int c = lane; c < ka; c += 32) pr[c] = first ? dr * rr[c] : dr * rr[c] + (T)beta[c] * pr[c];
    }
}

// partial sums of a*b over row slabs, active columns only
template <typename T>
__global__ void __launch_bounds__(256)
k_dot_partial(int n, int k, const T *__restrict__ A, const T *__restrict__ B, long ld,
              const int *__restrict__ nact, double *__restrict__ part, const T *__restrict__ wdiag = nullptr)
{
    __shared__ double sh[8][33];
    const int ka = nact ? *nact : k;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c = blockIdx.y * 32 + tx;
    const long r0 = (long)blockIdx.x * RED_ROWS, r1 = min((long)n, r0 + RED_ROWS);
    double s = 0;
    if (c < k && c < ka) {
        long r = r0 + ty;
        while (r < r1) {
            T run = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q, r += 8)
                if (r < r1) run = fma(A[r * ld + c], wdiag ? wdiag[r] * B[r * ld + c] : B[r * ld + c], run);
            s += (double)run;
        }
    }
    sh[ty][tx] = s;
    __syncthreads();
    if (ty == 0 && c < k) {
        double t = 0;
        for (int q = 0; q < 8; ++q) t += sh[q][tx];
        part[(long)blockIdx.x * k + c] = t;
    }
}

// x += alpha p, r -= alpha w (alpha = rho2/ptw) on active columns, with the
// partial sums of the new r.r
template <typename T>
__global__ void __launch_bounds__(256)
k_xr_update(int n, int k, T *__restrict__ X, T *__restrict__ R, const T *__restrict__ P,
            const T *__restrict__ W, long ld, const double *__restrict__ alpha,
            const int *__restrict__ nact, double *__restrict__ part, const T *__restrict__ dinv)
{
    __shared__ double sh[8][33];
    const int ka = *nact;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c = blockIdx.y * 32 + tx;
    const long r0 = (long)blockIdx.x * RED_ROWS, r1 = min((long)n, r0 + RED_ROWS);
    double s = 0;
    if (c < k && c < ka) {
        const T a = (T)alpha[c];
        long r = r0 + ty;
        while (r < r1) {
            T run = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q, r += 8) {
                if (r < r1) {
                    const long o = r * ld + c;
                    X[o] = X[o] + a * P[o];
                    const T rn = R[o] - a * W[o];
                    R[o] = rn;
                    run = fma(rn, dinv ? dinv[r] * rn : rn, run);   // r.z, z = D^-1 r or r
                }
            }
            s += (double)run;
        }
    }
    sh[ty][tx] = s;
    __syncthreads();
    if (ty == 0 && c < k && c < ka) {
        double t = 0;
        for (int q = 0; q < 8; ++q) t += sh[q][tx];
        part[(long)blockIdx.x * k + c] = t;
    }
}

// second stage of the per-column sums, one block per column: each thread adds a
// fixed strided subset of the row-slab partials, then a fixed tree (deterministic)
__global__ void __launch_bounds__(256)
k_colsum(int nblk, int k, const double *__restrict__ part, const int *__restrict__ nact, double *__restrict__ out)
{
    __shared__ double sh[256];
    const int c = blockIdx.x;
    if (nact && c >= *nact) return;
    double s = 0;
    for (int b = threadIdx.x; b < nblk; b += 256) s += part[(long)b * k + c];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = sh[0];
}

// ptw[c] (summed by k_colsum) for active c, and alpha[c] = rho2[c] / ptw[c]
__global__ void k_sum_active(int k, const int *__restrict__ nact, const double *__restrict__ ptw,
                             const double *__restrict__ rho2, double *__restrict__ alpha)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k || c >= *nact) return;
    alpha[c] = rho2[c] / ptw[c];
}

// initial residual norms: rho2 = column sums, err = sqrt(rho2), nact = k
__global__ void k_init_state(int k, const double *__restrict__ sums, double *rho2, double *err, int *nact)
{
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        rho2[c] = sums[c];
        err[c] = sqrt(sums[c]);
    }
    if (threadIdx.x == 0) *nact = k;
}

// end of a round: rho1 = rho2, rho2 = new r.r (active columns); recount over all columns
__global__ void k_finalize(int k, const double *__restrict__ sums, double *rho1, double *rho2,
                           const double *__restrict__ err, int *nact, double rate, double *beta)
{
    __shared__ int cnt;
    const int ka = *nact;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        if (c < ka) {
            const double s = sums[c];
            rho1[c] = rho2[c];
            rho2[c] = s;
            beta[c] = s / rho1[c];   // the next round's beta (src/gcge_cg.c:219)
        }
        const double lerr = sqrt(fabs(rho2[c]));
        if (lerr / err[c] >= rate) atomicAdd(&cnt, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) *nact = cnt;
}

// X += (double) D
__global__ void k_add_f2d(int n, int k, const float *__restrict__ D, long ldd, double *__restrict__ X, long ldx)
{
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) X[r * ldx + c] += (double)D[r * ldd + c];
}

// blocks of 8 warps for a warp-per-row loop, capped at 16 blocks per SM
static int row_grid(gcge_gpu_ctx *ctx, long rows)
{
    long g = (rows + 7) / 8, cap = (long)ctx->num_sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// partial-sum rows kept for the blocks of the FP32 long-row SpMM (past the
// cdiv(n, RED_ROWS) rows of the other kernels)
#define LONG_PART_ROWS 2048

extern "C" size_t gb_bcg_work_bytes(int n, int k, int precision)
{
    long ldk = (k + 3) & ~3;   // 16-byte rows for the vectorised SpMM
    size_t vec = precision ? sizeof(float) : sizeof(double);
    size_t nblk = (size_t)cdiv(n > 0 ? n : 1, RED_ROWS) + (precision ? LONG_PART_ROWS : 0);
    size_t blocks = 4 * (size_t)n * ldk * vec;  // R, X, P, W
    size_t state = (7 * (size_t)k + nblk * (size_t)k + 8) * sizeof(double) + 64;
    return blocks + state + 16 * 256;   // every sub-buffer is aligned to 256 bytes (10 of them)
}

// ---------------------------------------------------------------- FP32 rounds, fused
// The FP32 (mixed-precision) rounds (up to 256 columns) run on float4 kernels
// with fixed grids: block b always owns the same rows, so the per-block partial
// sums and their fixed-order column sums are deterministic. A round is five
// launches -- p update, SpMM with the p.w partials in its epilogue, alpha, x/r
// update with the r.r partials, beta and the active count -- plus a sixth for
// matrices with rows longer than GB_LONG_ROW (their SpMM rows, a block each).
#define VB_THREADS 256

// Blocks of a grid-stride kernel of the fused rounds: the blocks that are resident
// at once (its occupancy at VB_THREADS threads, times the SMs) divided over the
// column tiles, so that every block is in the first wave -- a grid one block per
// SM past that leaves those blocks running alone after the others finish.
static int vec_blocks(gcge_gpu_ctx *ctx, const void *fn, int n, int ctiles)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, VB_THREADS, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    long g = cdiv(n > 0 ? n : 1, RED_ROWS), cap = (long)ctx->num_sms * per_sm / (ctiles > 0 ? ctiles : 1);
    if (cap < 1) cap = 1;
    return (int)(g < cap ? g : cap);
}

// sum the per-thread column partials s[4] (thread (rs, cg) holds columns
// c0 + 4 cg .. +3 of its row slot) over the row slots in a fixed order; the block's
// partials of the kact active columns go to row blockIdx.x of part (row stride k,
// the layout that the column-sum kernels read)
template <int SLOTS, int COLS>
__device__ __forceinline__ void vb_block_reduce(const double s[4], int slot, int cg, int c0, int kact, int k,
                                                double *part)
{
    __shared__ double red[SLOTS][COLS + 1];
#pragma unroll
    for (int q = 0; q < 4; ++q) red[slot][4 * cg + q] = s[q];
    __syncthreads();
    for (int c = threadIdx.x; c < COLS; c += blockDim.x) {
        double t = 0;
        for (int r = 0; r < SLOTS; ++r) t += red[r][c];
        if (c0 + c < kact) part[(long)blockIdx.x * k + c0 + c] = t;
    }
}

// The vector kernels of the fused rounds: TPR threads per row (1, 2, 4, 8 or 16,
// the fewest whose float4 groups cover k, 16 with 64-column tiles over blockIdx.y
// beyond 64 columns), 4 columns per thread, 256 / TPR rows per block pass; a warp
// reads 32 TPR-thread row segments, one contiguous run when 4 TPR = ld.

// p = r + beta p (p = r on the first round) on the active columns
template <int TPR>
__global__ void __launch_bounds__(VB_THREADS)
k_pupdate_v(int n, int k, const float *__restrict__ R, float *__restrict__ P, long ld,
            const double *__restrict__ beta, const int *__restrict__ nact, int first,
            const float *__restrict__ dinv)
{
    constexpr int RPB = VB_THREADS / TPR;
    const int ka = min(*nact, k);
    const int cg = threadIdx.x % TPR, rs = threadIdx.x / TPR;
    const int c0 = blockIdx.y * 64 + 4 * cg;
    if (c0 >= ka) return;
    float b[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) b[q] = (!first && c0 + q < ka) ? (float)beta[c0 + q] : 0.f;
    const bool full = c0 + 4 <= ka;
    for (long r = (long)blockIdx.x * RPB + rs; r < n; r += (long)gridDim.x * RPB) {
        float4 rv = *reinterpret_cast<const float4 *>(R + r * ld + c0);
        if (dinv) {                                // z = D^-1 r (Jacobi)
            const float dr = dinv[r];
            rv.x *= dr; rv.y *= dr; rv.z *= dr; rv.w *= dr;
        }
        float4 *pp = reinterpret_cast<float4 *>(P + r * ld + c0);
        if (first) {                               // p = r: the old p (uninitialised) is not read
            if (full) {
                *pp = rv;
            } else {
                float *pe = reinterpret_cast<float *>(pp);
                const float *re = &rv.x;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (c0 + q < ka) pe[q] = re[q];
            }
            continue;
        }
        float4 pv = *pp;
        if (full) {
            pv.x = rv.x + b[0] * pv.x; pv.y = rv.y + b[1] * pv.y;
            pv.z = rv.z + b[2] * pv.z; pv.w = rv.w + b[3] * pv.w;
        } else {
            float *pe = &pv.x;
            const float *re = &rv.x;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (c0 + q < ka) pe[q] = re[q] + b[q] * pe[q];
        }
        *pp = pv;
    }
}

// x += alpha p, r -= alpha w on the active columns, with block partials of r.r
// (FP32 products summed over runs of 8 rows, the runs summed in FP64)
template <int TPR>
__global__ void __launch_bounds__(VB_THREADS)
k_xr_update_v(int n, int k, float *__restrict__ X, float *__restrict__ R, const float *__restrict__ P,
              const float *__restrict__ W, long ld, const double *__restrict__ alpha, const int *__restrict__ nact,
              double *__restrict__ part, const float *__restrict__ dinv)
{
    constexpr int RPB = VB_THREADS / TPR;
    const int ka = min(*nact, k);
    const int cg = threadIdx.x % TPR, rs = threadIdx.x / TPR;
    const int c0 = blockIdx.y * 64 + 4 * cg;
    double s[4] = {0, 0, 0, 0};
    if (c0 < ka) {
        float a[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = c0 + q < ka ? (float)alpha[c0 + q] : 0.f;
        float run[4] = {0, 0, 0, 0};
        int cnt = 0;
        for (long r = (long)blockIdx.x * RPB + rs; r < n; r += (long)gridDim.x * RPB) {
            const long o = r * ld + c0;
            float4 xv = *reinterpret_cast<const float4 *>(X + o);
            float4 rv = *reinterpret_cast<const float4 *>(R + o);
            const float4 pv = *reinterpret_cast<const float4 *>(P + o);
            const float4 wv = *reinterpret_cast<const float4 *>(W + o);
            float *xe = &xv.x, *re = &rv.x;
            const float *pe = &pv.x, *we = &wv.x;
            const float dr = dinv ? dinv[r] : 1.0f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                xe[q] = xe[q] + a[q] * pe[q];      // a = 0 leaves inactive columns unchanged
                re[q] = re[q] - a[q] * we[q];
                run[q] = fmaf(re[q], dr * re[q], run[q]);   // r.z, z = D^-1 r or r
            }
            *reinterpret_cast<float4 *>(X + o) = xv;
            *reinterpret_cast<float4 *>(R + o) = rv;
            if (++cnt == 8) {
#pragma unroll
                for (int q = 0; q < 4; ++q) { s[q] += (double)run[q]; run[q] = 0.f; }
                cnt = 0;
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) s[q] += (double)run[q];
    }
    vb_block_reduce<RPB, 4 * TPR>(s, rs, cg, blockIdx.y * 64, ka, k, part);
}

// The long rows (the list lrows, nlong of them, longest first: a power-law
// graph's hubs reach thousands of entries) of W = A P: each block takes one row
// at a time with all 256 / L lane groups, group g summing the row's entries
// g L .. + L - 1 modulo 256, and the group sums are added in shared memory in
// group order. Rows are dealt to the blocks in snake order (round r: block b
// takes list entry r G + b, or r G + G - 1 - b for odd r), so the blocks carry
// nearly equal entry counts. Column c's p.w partial is summed in FP64 by thread
// c and written to row part_row0 + blockIdx.x of part.
template <int L, int NV>
__global__ void __launch_bounds__(VB_THREADS)
k_spmm32_long(const int *__restrict__ rp, const int *__restrict__ ci, const float *__restrict__ val,
              const float *__restrict__ P, float *__restrict__ W, long ld, int k, const int *__restrict__ nact,
              double *__restrict__ part, int part_row0, const int *__restrict__ lrows, int nlong)
{
    constexpr int RPB = VB_THREADS / L, COLS = 4 * L * NV, UNR = 4;
    __shared__ float rs[RPB * COLS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / L, sl = lane % L;
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (sub * L));
    const int slot = warp * (32 / L) + sub;
    const int kact = min(*nact, k), G = gridDim.x, b = blockIdx.x;
    double pw = 0.0;
    for (int r = 0; kact > 0; ++r) {
        const long li = (long)r * G + ((r & 1) ? G - 1 - b : b);
        if (li >= nlong) break;
        const long row = lrows[li];
        const int beg = rp[row], end = rp[row + 1];
        float acc[4 * NV];
#pragma unroll
        for (int q = 0; q < 4 * NV; ++q) acc[q] = 0.f;
        for (int base = beg + slot * L; base < end; base += RPB * L) {
            const int e = base + sl;
            int j = 0;
            float a = 0.f;
            if (e < end) { j = __ldg(ci + e); a = __ldg(val + e); }
            const int m = min(L, end - base);
#pragma unroll UNR
            for (int t = 0; t < m; ++t) {
                const int jj = __shfl_sync(gmask, j, t, L);
                const float aa = __shfl_sync(gmask, a, t, L);
                const float *xr = P + (long)jj * ld + 4 * sl;
#pragma unroll
                for (int v = 0; v < NV; ++v)
                    if (4 * sl + 4 * L * v < kact) {
                        const float4 xv = __ldg(reinterpret_cast<const float4 *>(xr + 4 * L * v));
                        acc[4 * v + 0] = fmaf(aa, xv.x, acc[4 * v + 0]);
                        acc[4 * v + 1] = fmaf(aa, xv.y, acc[4 * v + 1]);
                        acc[4 * v + 2] = fmaf(aa, xv.z, acc[4 * v + 2]);
                        acc[4 * v + 3] = fmaf(aa, xv.w, acc[4 * v + 3]);
                    }
            }
        }
        __syncthreads();                                      // the previous row's sums are read
#pragma unroll
        for (int v = 0; v < NV; ++v)
#pragma unroll
            for (int q = 0; q < 4; ++q) rs[slot * COLS + 4 * sl + 4 * L * v + q] = acc[4 * v + q];
        __syncthreads();
        const int c = threadIdx.x;
        if (c < COLS && c < kact) {
            float t = 0.f;
            for (int g = 0; g < RPB; ++g) t += rs[g * COLS + c];
            W[row * ld + c] = t;
            pw += (double)(P[row * ld + c] * t);
        }
    }
    if (threadIdx.x < COLS && (int)threadIdx.x < kact) part[(long)(part_row0 + b) * k + threadIdx.x] = pw;
}

// W = A P (FP32, the first nact columns) and block partials of p.w: L lanes per
// row, NV float4 column groups per lane (lane l owns columns 4l + 4Lv .. +3, so
// that each group load of the L lanes reads one contiguous 16L-byte run), 256 / L
// rows per block pass; grid-stride over rows (measured faster than contiguous row
// ranges per block on the Q1 cube). Rows longer than lim are skipped (the long-row
// kernel above has them). NV = 2 halves the shuffles and address arithmetic per
// FMA. The gathers of P rows are L2 hits whose latency bounds the kernel, so four
// entries' loads are in flight per lane (64 registers, 4 blocks per SM: 8% faster
// at fem96 k = 64 than two at 48 registers and 5 blocks). The p.w products are
// summed in FP32 over runs of 8 rows of a row slot and the runs added in FP64 to
// the slot's shared-memory partials (the thread's own entries: no atomics, fixed
// order).
template <int L, int NV>
__global__ void __launch_bounds__(VB_THREADS, 4)                  // 64 registers: 4 blocks per SM
k_spmm32_dot(int n, const int *__restrict__ rp, const int *__restrict__ ci, const float *__restrict__ val,
             const float *__restrict__ P, float *__restrict__ W, long ld, int k, const int *__restrict__ nact,
             double *__restrict__ part, int lim)
{
    constexpr int RPB = VB_THREADS / L, COLS = 4 * L * NV, UNR = 4;
    __shared__ double red[RPB][COLS + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / L, sl = lane % L;
    const unsigned gmask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (sub * L));
    const int slot = warp * (32 / L) + sub;
    const int kact = min(*nact, k);
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int q = 0; q < 4; ++q) red[slot][4 * sl + 4 * L * v + q] = 0.0;
    float run[4 * NV];
#pragma unroll
    for (int q = 0; q < 4 * NV; ++q) run[q] = 0.f;
    int cnt = 0;
    if (kact > 0)
        for (long row = (long)blockIdx.x * RPB + slot; row < n; row += (long)gridDim.x * RPB) {
            const int beg = rp[row], end = rp[row + 1];
            if (end - beg > lim) continue;                    // a long row: k_spmm32_long
            float acc[4 * NV];
#pragma unroll
            for (int q = 0; q < 4 * NV; ++q) acc[q] = 0.f;
            for (int base = beg; base < end; base += L) {
                const int e = base + sl;
                int j = 0;
                float a = 0.f;
                if (e < end) { j = __ldg(ci + e); a = __ldg(val + e); }
                const int m = min(L, end - base);
#pragma unroll UNR
                for (int t = 0; t < m; ++t) {
                    const int jj = __shfl_sync(gmask, j, t, L);
                    const float aa = __shfl_sync(gmask, a, t, L);
                    const float *xr = P + (long)jj * ld + 4 * sl;
#pragma unroll
                    for (int v = 0; v < NV; ++v)
                        if (4 * sl + 4 * L * v < kact) {
                            const float4 xv = __ldg(reinterpret_cast<const float4 *>(xr + 4 * L * v));
                            acc[4 * v + 0] = fmaf(aa, xv.x, acc[4 * v + 0]);
                            acc[4 * v + 1] = fmaf(aa, xv.y, acc[4 * v + 1]);
                            acc[4 * v + 2] = fmaf(aa, xv.z, acc[4 * v + 2]);
                            acc[4 * v + 3] = fmaf(aa, xv.w, acc[4 * v + 3]);
                        }
                }
            }
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                const int c = 4 * sl + 4 * L * v;
                if (c < kact) {
                    const long o = row * ld + c;
                    const float4 pv = *reinterpret_cast<const float4 *>(P + o);
                    const float *pe = &pv.x;
                    float4 *wp = reinterpret_cast<float4 *>(W + o);
                    if (c + 4 <= kact) {
                        *wp = make_float4(acc[4 * v], acc[4 * v + 1], acc[4 * v + 2], acc[4 * v + 3]);
                    } else {
                        float *we = reinterpret_cast<float *>(wp);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (c + q < kact) we[q] = acc[4 * v + q];
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (c + q < kact) run[4 * v + q] = fmaf(pe[q], acc[4 * v + q], run[4 * v + q]);
                }
            }
            if (++cnt == 8) {
#pragma unroll
                for (int v = 0; v < NV; ++v)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        red[slot][4 * sl + 4 * L * v + q] += (double)run[4 * v + q];
                        run[4 * v + q] = 0.f;
                    }
                cnt = 0;
            }
        }
#pragma unroll
    for (int v = 0; v < NV; ++v)
#pragma unroll
        for (int q = 0; q < 4; ++q) red[slot][4 * sl + 4 * L * v + q] += (double)run[4 * v + q];
    __syncthreads();
    for (int c = threadIdx.x; c < COLS; c += blockDim.x) {
        double t = 0;
        for (int r = 0; r < RPB; ++r) t += red[r][c];
        if (c < kact) part[(long)blockIdx.x * k + c] = t;
    }
}

// column sums of the block partials (one block per active column, fixed order)
// and alpha[c] = rho2[c] / ptw[c]
__global__ void __launch_bounds__(256)
k_colsum_alpha(int nblk, int k, const double *__restrict__ part, const int *__restrict__ nact,
               const double *__restrict__ rho2, double *__restrict__ ptw, double *__restrict__ alpha)
{
    __shared__ double sh[256];
    const int c = blockIdx.x;
    if (c >= *nact) return;
    double s = 0;
    for (int b = threadIdx.x; b < nblk; b += 256) s += part[(long)b * k + c];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ptw[c] = sh[0];
        alpha[c] = rho2[c] / sh[0];
    }
}

// column sums of the r.r partials (a warp per column, fixed order), then the
// end-of-round update of k_finalize in the same block
__global__ void __launch_bounds__(1024)
k_colsum_finalize(int nblk, int k, const double *__restrict__ part, double *sums, double *rho1, double *rho2,
                  const double *__restrict__ err, int *nact, double rate, double *beta)
{
    __shared__ int cnt;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ka = *nact;
    if (threadIdx.x == 0) cnt = 0;
    for (int c = warp; c < ka; c += 32) {
        double s = 0;
        for (int b = lane; b < nblk; b += 32) s += part[(long)b * k + c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) sums[c] = s;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        if (c < ka) {
            const double s = sums[c];
            rho1[c] = rho2[c];
            rho2[c] = s;
            beta[c] = s / rho1[c];   // the next round's beta (src/gcge_cg.c:219)
        }
        const double lerr = sqrt(fabs(rho2[c]));
        if (lerr / err[c] >= rate) atomicAdd(&cnt, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) *nact = cnt;
}

typedef void (*pupdate_fn)(int, int, const float *, float *, long, const double *, const int *, int,
                           const float *);
typedef void (*spmm32_fn)(int, const int *, const int *, const float *, const float *, float *, long, int,
                          const int *, double *, int);
typedef void (*spmm32l_fn)(const int *, const int *, const float *, const float *, float *, long, int, const int *,
                           double *, int, const int *, int);
typedef void (*xr_fn)(int, int, float *, float *, const float *, const float *, long, const double *, const int *,
                      double *, const float *);

static int bcg_rounds32(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, float *R, float *X, float *P, float *W, long ld,
                        const gb_bcg_args *a, bcg_state *s)
{
    const int n = a->n, k = a->k;
    if (k > 256 || !A->v32) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    const int ctiles = (k + 63) / 64;
    // vector kernels: threads per row whose float4 groups cover k; SpMM: L lanes per
    // row with NV float4 groups each, 4 L NV >= k
    const int tpr = k <= 4 ? 1 : (k <= 8 ? 2 : (k <= 16 ? 4 : (k <= 32 ? 8 : 16)));
    const pupdate_fn pup = tpr == 1 ? k_pupdate_v<1> : tpr == 2 ? k_pupdate_v<2> : tpr == 4 ? k_pupdate_v<4>
                         : tpr == 8 ? k_pupdate_v<8> : k_pupdate_v<16>;
    const xr_fn xru = tpr == 1 ? k_xr_update_v<1> : tpr == 2 ? k_xr_update_v<2> : tpr == 4 ? k_xr_update_v<4>
                    : tpr == 8 ? k_xr_update_v<8> : k_xr_update_v<16>;
    const spmm32_fn spm = k <= 4 ? k_spmm32_dot<1, 1> : k <= 8 ? k_spmm32_dot<2, 1> : k <= 16 ? k_spmm32_dot<4, 1>
                        : k <= 32 ? k_spmm32_dot<4, 2> : k <= 64 ? k_spmm32_dot<8, 2>
                        : k <= 128 ? k_spmm32_dot<16, 2> : k_spmm32_dot<32, 2>;
    const int Gp = vec_blocks(ctx, (const void *)pup, n, ctiles);
    const int Gs = vec_blocks(ctx, (const void *)spm, n, 1);
    const int Gx = vec_blocks(ctx, (const void *)xru, n, ctiles);
    // rows longer than GB_LONG_ROW: a launch of their own before the grid-stride
    // product (one wave of blocks over the sorted list); its p.w partials follow
    // the Gs rows of the other launch in part, which holds LONG_PART_ROWS rows
    // past cdiv(n, RED_ROWS)
    const spmm32l_fn spl = k <= 4 ? k_spmm32_long<1, 1> : k <= 8 ? k_spmm32_long<2, 1> : k <= 16 ? k_spmm32_long<4, 1>
                         : k <= 32 ? k_spmm32_long<4, 2> : k <= 64 ? k_spmm32_long<8, 2>
                         : k <= 128 ? k_spmm32_long<16, 2> : k_spmm32_long<32, 2>;
    int Gl = 0;
    if (A->nlong > 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)spl, VB_THREADS, 0) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        const long room = cdiv(n, RED_ROWS) + LONG_PART_ROWS - (long)Gs, cap = (long)ctx->num_sms * per_sm;
        long g = A->nlong < cap ? A->nlong : cap;
        Gl = (int)(g < room ? g : room);
        if (Gl < 0) Gl = 0;
    }
    const int lim = Gl > 0 ? GB_LONG_ROW : 0x7fffffff;
    const double lbytes = Gl > 0 ? 8.0 * A->nnz_long + 12.0 * A->nlong * k : 0.0;
    for (int it = 1; it < a->max_it; ++it) {
        GB_PROF(ctx, GB_K_BCGVEC, 12.0 * n * k, 2.0 * n * k);
        GB_LAUNCH(ctx, pup, dim3(Gp, ctiles), VB_THREADS, 0, n, k, R, P, ld, s->beta, s->nact, it == 1, a->dinv32);
        ctx->spmm_launches++;
        if (Gl > 0) {
            GB_PROF(ctx, GB_K_SPMM32, lbytes, 2.0 * A->nnz_long * k + 2.0 * A->nlong * k);
            GB_LAUNCH(ctx, spl, Gl, VB_THREADS, 0, A->rp, A->ci, A->v32, P, W, ld, k, s->nact, s->part, Gs, A->lrows,
                      A->nlong);
        }
        GB_PROF(ctx, GB_K_SPMM32, 8.0 * A->nnz + 4.0 * (A->n + 1) + 12.0 * A->n * k - lbytes,
                2.0 * (A->nnz - (Gl > 0 ? A->nnz_long : 0)) * k + 2.0 * A->n * k);
        GB_LAUNCH(ctx, spm, Gs, VB_THREADS, 0, n, A->rp, A->ci, A->v32, P, W, ld, k, s->nact, s->part, lim);
        GB_LAUNCH(ctx, k_colsum_alpha, k, 256, 0, Gs + Gl, k, s->part, s->nact, s->rho2, s->ptw, s->alpha);
        GB_PROF(ctx, GB_K_BCGVEC, 24.0 * n * k, 6.0 * n * k);
        GB_LAUNCH(ctx, xru, dim3(Gx, ctiles), VB_THREADS, 0, n, k, X, R, P, W, ld, s->alpha, s->nact, s->part,
                  a->dinv32);
        GB_LAUNCH(ctx, k_colsum_finalize, 1, 1024, 0, Gx, k, s->part, s->sums, s->rho1, s->rho2, s->err, s->nact,
                  a->rate, s->beta);
    }
    return GCGE_GPU_OK;
}

template <typename T>
static int bcg_rounds(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, T *R, T *X, T *P, T *W, long ld,
                      const gb_bcg_args *a, bcg_state *s)
{
    const int n = a->n, k = a->k, nblk = cdiv(n > 0 ? n : 1, RED_ROWS);
    dim3 rgrid(nblk, (k + 31) / 32);
    const double es = sizeof(T);
    const T *dv = sizeof(T) == sizeof(double) ? (const T *)(const void *)a->dinv : (const T *)(const void *)a->dinv32;
    for (int it = 1; it < a->max_it; ++it) {
        GB_PROF(ctx, GB_K_BCGVEC, 3.0 * es * n * k, 2.0 * n * k);
        GB_LAUNCH(ctx, k_pupdate<T>, row_grid(ctx, n), 256, 0, n, k, R, P, ld, s->beta, s->nact, it == 1, dv);
        int st;
        if (sizeof(T) == sizeof(double))
            st = gb_spmm(ctx, A, (const double *)P, ld, (double *)W, ld, k, 1.0, nullptr, 0.0, s->nact);
        else
            st = gb_spmm32(ctx, A, (const float *)P, ld, (float *)W, ld, k, s->nact);
        if (st) return st;
        GB_PROF(ctx, GB_K_BCGVEC, 2.0 * es * n * k, 2.0 * n * k);
        GB_LAUNCH(ctx, k_dot_partial<T>, rgrid, 256, 0, n, k, P, W, ld, s->nact, s->part);
        GB_LAUNCH(ctx, k_colsum, k, 256, 0, nblk, k, s->part, s->nact, s->ptw);
        GB_LAUNCH(ctx, k_sum_active, (k + 127) / 128, 128, 0, k, s->nact, s->ptw, s->rho2, s->alpha);
        GB_PROF(ctx, GB_K_BCGVEC, 6.0 * es * n * k, 6.0 * n * k);
        GB_LAUNCH(ctx, k_xr_update<T>, rgrid, 256, 0, n, k, X, R, P, W, ld, s->alpha, s->nact, s->part, dv);
        GB_LAUNCH(ctx, k_colsum, k, 256, 0, nblk, k, s->part, s->nact, s->sums);
        GB_LAUNCH(ctx, k_finalize, 1, 256, 0, k, s->sums, s->rho1, s->rho2, s->err, s->nact, a->rate, s->beta);
    }
    return GCGE_GPU_OK;
}

extern "C" int gb_bcg(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, double *RHS, long ldr, double *X, long ldx,
                      const gb_bcg_args *a, void *work, size_t work_bytes)
{
    const int n = a->n, k = a->k;
    if (k <= 0 || n <= 0) return GCGE_GPU_OK;
    if (work_bytes < gb_bcg_work_bytes(n, k, a->precision)) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (a->precision && !A->v32) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    const long ld = (k + 3) & ~3;
    const int nblk = cdiv(n, RED_ROWS);
    char *w = (char *)work;
    size_t vec = a->precision ? sizeof(float) : sizeof(double);
    auto take = [&](size_t bytes) { char *p = w; w += (bytes + 255) & ~(size_t)255; return (void *)p; };
    bcg_state s;
    s.rho1 = (double *)take(sizeof(double) * k);
    s.rho2 = (double *)take(sizeof(double) * k);
    s.err = (double *)take(sizeof(double) * k);
    s.ptw = (double *)take(sizeof(double) * k);
    s.alpha = (double *)take(sizeof(double) * k);
    s.beta = (double *)take(sizeof(double) * k);
    s.sums = (double *)take(sizeof(double) * k);
    s.part = (double *)take(sizeof(double) * (size_t)(nblk + (a->precision ? LONG_PART_ROWS : 0)) * k);
    s.nact = (int *)take(64);
    dim3 rgrid(nblk, (k + 31) / 32);
    if (a->precision == 0) {
        double *P = (double *)take((size_t)n * ld * vec);
        double *W = (double *)take((size_t)n * ld * vec);
        (void)W;
        // R = RHS - A X, in place in RHS (the reference overwrites RHS with the residual)
        int st = a->rhs_is_residual ? 0 : gb_spmm(ctx, A, X, ldx, RHS, ldr, k, -1.0, nullptr, 1.0, nullptr);
        if (st) return st;
        // P and W use the compact ld; R and X keep their own ld through the copies below
        if (ldr == ld && ldx == ld) {
            GB_LAUNCH(ctx, k_dot_partial<double>, rgrid, 256, 0, n, k, RHS, RHS, ld, (const int *)nullptr, s.part,
                      a->dinv);
            GB_LAUNCH(ctx, k_colsum, k, 256, 0, nblk, k, s.part, (const int *)nullptr, s.sums);
            GB_LAUNCH(ctx, k_init_state, 1, 256, 0, k, s.sums, s.rho2, s.err, s.nact);
            return bcg_rounds<double>(ctx, A, RHS, X, P, W, ld, a, &s);
        }
        // general leading dimensions: stage R and X in compact blocks
        double *R = (double *)take((size_t)n * ld * vec);
        double *Xc = (double *)take((size_t)n * ld * vec);
        if ((size_t)(w - (char *)work) > work_bytes) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
        if ((st = gb_axpby(ctx, n, k, 1.0, RHS, ldr, 0.0, R, ld))) return st;
        if ((st = gb_axpby(ctx, n, k, 1.0, X, ldx, 0.0, Xc, ld))) return st;
        GB_LAUNCH(ctx, k_dot_partial<double>, rgrid, 256, 0, n, k, R, R, ld, (const int *)nullptr, s.part, a->dinv);
        GB_LAUNCH(ctx, k_colsum, k, 256, 0, nblk, k, s.part, (const int *)nullptr, s.sums);
            GB_LAUNCH(ctx, k_init_state, 1, 256, 0, k, s.sums, s.rho2, s.err, s.nact);
        if ((st = bcg_rounds<double>(ctx, A, R, Xc, P, W, ld, a, &s))) return st;
        if ((st = gb_axpby(ctx, n, k, 1.0, Xc, ld, 0.0, X, ldx))) return st;
        return gb_axpby(ctx, n, k, 1.0, R, ld, 0.0, RHS, ldr);
    }
    // Mixed precision as defect correction: the residual r0 = RHS - A X is formed in
    // FP64, block CG runs in FP32 on A D = r0 from D = 0, and X += D in FP64. The
    // iteration is the reference's in exact arithmetic, while the correction D, not
    // the whole solution, carries the FP32 rounding.
    float *R = (float *)take((size_t)n * ld * vec);
    float *D = (float *)take((size_t)n * ld * vec);
    float *P = (float *)take((size_t)n * ld * vec);
    float *W = (float *)take((size_t)n * ld * vec);
    if ((size_t)(w - (char *)work) > work_bytes) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    int st;
    if (!a->rhs_is_residual && (st = gb_spmm(ctx, A, X, ldx, RHS, ldr, k, -1.0, nullptr, 1.0, nullptr))) return st;
    if ((st = gb_convert_d2f(ctx, n, k, RHS, ldr, R, ld))) return st;
    if (cudaMemsetAsync(D, 0, (size_t)n * ld * sizeof(float), ctx->stream) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    GB_LAUNCH(ctx, k_dot_partial<float>, rgrid, 256, 0, n, k, R, R, ld, (const int *)nullptr, s.part, a->dinv32);
    GB_LAUNCH(ctx, k_colsum, k, 256, 0, nblk, k, s.part, (const int *)nullptr, s.sums);
    GB_LAUNCH(ctx, k_init_state, 1, 256, 0, k, s.sums, s.rho2, s.err, s.nact);
    if ((st = k <= 256 ? bcg_rounds32(ctx, A, R, D, P, W, ld, a, &s) : bcg_rounds<float>(ctx, A, R, D, P, W, ld, a, &s)))
        return st;
    GB_LAUNCH(ctx, k_add_f2d, row_grid(ctx, n), 256, 0, n, k, D, ld, X, ldx);
    return a->residual_unused ? GCGE_GPU_OK : gb_convert_f2d(ctx, n, k, R, ld, RHS, ldr);
}

__global__ void k_axpy32(int n, int k, float a, const float *__restrict__ X, float *__restrict__ Y, long ld)
{
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) Y[r * ld + c] += a * X[r * ld + c];
}

extern "C" int gb_axpy32(gcge_gpu_ctx *ctx, int n, int k, float a, const float *X, float *Y, long ld)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_axpy32, row_grid(ctx, n), 256, 0, n, k, a, X, Y, ld);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- Jacobi preconditioner
// dinv[r] = 1 / A[r, r] (1 where the row has no nonzero diagonal entry), FP64 and FP32
__global__ void k_diag_inv(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                           const double *__restrict__ v, double *__restrict__ dinv, float *__restrict__ dinv32)
{
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
        double dg = 0.0;
        for (int e = rp[r]; e < rp[r + 1]; ++e)
            if (ci[e] == r) dg += v[e];
        const double di = dg != 0.0 ? 1.0 / dg : 1.0;
        dinv[r] = di;
        dinv32[r] = (float)di;
    }
}

extern "C" int gb_mat_dinv(gcge_gpu_ctx *ctx, gcge_gpu_mat *A)
{
    if (A->dinv) return GCGE_GPU_OK;
    const size_t n = (size_t)(A->n > 0 ? A->n : 1);
    if (cudaMalloc(&A->dinv, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&A->dinv32, sizeof(float) * n) != cudaSuccess) {
        cudaFree(A->dinv);
        A->dinv = nullptr;
        A->dinv32 = nullptr;
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    GB_LAUNCH(ctx, k_diag_inv, row_grid(ctx, A->n / 8 + 1), 256, 0, A->n, A->rp, A->ci, A->v, A->dinv, A->dinv32);
    return GCGE_GPU_OK;
}
