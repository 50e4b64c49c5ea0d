// gb_blas.cu -- HBM-streaming kernels of the GCGE hot path on GB300 (sm_103a).
//
//  * CSR SpMM against row-major multivector blocks (FP64 and FP32 values):
//    one warp per (row, 64-column chunk); the row's (column, value) pairs are
//    loaded once per 32 entries with coalesced loads and broadcast by shuffles,
//    and every nonzero gathers one contiguous block row of X.
//  * AXPBY / gathers / conversions: grid-stride element kernels.
//  * Per-column dot products, residual norms and tall-skinny Gram products:
//    deterministic two-stage reductions (fixed partition of the rows, partials
//    in scratch, fixed-order second stage), so results do not depend on timing.
//  * Linear combinations X*C: 64-row x 32-column output tiles with X and C
//    staged in shared memory.
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "gb_internal.h"

#define FULL 0xffffffffu

static inline int ceil_div_l(long a, long b) { return (int)((a + b - 1) / b); }

#define GB_LAUNCH(ctx, kern, grid, block, smem, ...)                                   \
    do {                                                                               \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                 \
        (ctx)->launches++;                                                             \
        if ((ctx)->prof) gb_prof_end(ctx);                                             \
        int _st = gb_check_launch(ctx);                                                \
        if (_st) return _st;                                                           \
    } while (0)

// profile the next launch (no-op unless profiling is enabled on the context)
#define GB_PROF(ctx, cls, bytes, flops) \
    do { if ((ctx)->prof) gb_prof_begin((ctx), (cls), (bytes), (flops)); } while (0)

// ---------------------------------------------------------------- SpMM
// Y[row, c] = alpha * alpha_col[c] * sum_j A[row, j] X[j, c] + beta * Y[row, c]
template <typename VT, typename XT, typename AT>
__global__ void __launch_bounds__(256)
k_spmm(int n, const int *__restrict__ rp, const int *__restrict__ ci, const VT *__restrict__ val,
       const XT *__restrict__ X, long ldx, XT *__restrict__ Y, long ldy, int k, AT alpha,
       const double *__restrict__ alpha_col, AT beta, const int *__restrict__ ncols_dev)
{
    const int lane = threadIdx.x & 31;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nchunks = (k + 63) >> 6;
    if (warp >= (long)n * nchunks) return;                 // warp-uniform
    int kact = k;
    if (ncols_dev) kact = min(k, *ncols_dev);
    const int row = (int)(warp / nchunks);
    const int chunk = (int)(warp - (long)row * nchunks);
    const int c0 = chunk * 64 + lane, c1 = c0 + 32;
    if (chunk * 64 >= kact) return;                        // warp-uniform
    const bool h0 = c0 < kact, h1 = c1 < kact;
    AT acc0 = 0, acc1 = 0;
    const int beg = rp[row], end = rp[row + 1];
    for (int base = beg; base < end; base += 32) {
        const int e = base + lane;
        int j = 0;
        VT a = 0;
        if (e < end) { j = __ldg(ci + e); a = __ldg(val + e); }
        const int cnt = min(32, end - base);
        for (int t = 0; t < cnt; ++t) {
            const int jj = __shfl_sync(FULL, j, t);
            const AT aa = (AT)__shfl_sync(FULL, a, t);
            const XT *xr = X + (long)jj * ldx;
            if (h0) acc0 = fma(aa, (AT)__ldg(xr + c0), acc0);
            if (h1) acc1 = fma(aa, (AT)__ldg(xr + c1), acc1);
        }
    }
    XT *yr = Y + (long)row * ldy;
    if (h0) {
        AT s = alpha * (alpha_col ? (AT)alpha_col[c0] : (AT)1);
        yr[c0] = (XT)(beta == (AT)0 ? s * acc0 : s * acc0 + beta * (AT)yr[c0]);
    }
    if (h1) {
        AT s = alpha * (alpha_col ? (AT)alpha_col[c1] : (AT)1);
        yr[c1] = (XT)(beta == (AT)0 ? s * acc1 : s * acc1 + beta * (AT)yr[c1]);
    }
}

// Vectorised SpMM: a group of L lanes (L = 4, 8, 16 or 32) owns one row and VW =
// 16 / sizeof(T) consecutive columns per lane, so each nonzero gathers its block
// row of X with one 16-byte load per lane; 32 / L rows per warp. The group loads
// up to L (column, value) pairs at once and broadcasts them with group-masked
// shuffles. AL: X and ldx 16-byte aligned (otherwise the slice is read element
// by element, for column ranges that start at an odd column).
template <typename T> struct vec16;
template <> struct vec16<float> { typedef float4 type; };
template <> struct vec16<double> { typedef double2 type; };

template <typename T, int L, bool AL = true>
__global__ void __launch_bounds__(256)
k_spmm_vec(int n, const int *__restrict__ rp, const int *__restrict__ ci, const T *__restrict__ val,
           const T *__restrict__ X, long ldx, T *__restrict__ Y, long ldy, int k, T alpha,
           const double *__restrict__ alpha_col, T beta, const int *__restrict__ ncols_dev)
{
    typedef typename vec16<T>::type V;
    constexpr int VW = 16 / sizeof(T);
    constexpr int RPW = 32 / L;
    const int lane = threadIdx.x & 31;
    const int sub = lane / L, sl = lane % L;
    const unsigned gmask = (L == 32) ? FULL : (((1u << L) - 1u) << (sub * L));
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long row = warp * RPW + sub;
    int kact = k;
    if (ncols_dev) kact = min(k, *ncols_dev);
    if (row >= n || kact <= 0) return;                    // uniform within the row group
    const int beg = rp[row], end = rp[row + 1];
    for (int c0 = 0; c0 < kact; c0 += L * VW) {
        const int c = c0 + sl * VW;
        const bool full = c + VW <= kact;
        T acc[VW];
#pragma unroll
        for (int q = 0; q < VW; ++q) acc[q] = 0;
        for (int base = beg; base < end; base += L) {
            const int e = base + sl;
            int j = 0;
            T a = 0;
            if (e < end) { j = __ldg(ci + e); a = __ldg(val + e); }
            const int cnt = min(L, end - base);
#pragma unroll 4
            for (int t = 0; t < cnt; ++t) {
                const int jj = __shfl_sync(gmask, j, t, L);
                const T aa = __shfl_sync(gmask, a, t, L);
                const T *xr = X + (long)jj * ldx + c;
                if (full) {
                    if (AL) {
                        const V xv = __ldg(reinterpret_cast<const V *>(xr));
                        const T *xs = reinterpret_cast<const T *>(&xv);
#pragma unroll
                        for (int q = 0; q < VW; ++q) acc[q] = fma(aa, xs[q], acc[q]);
                    } else {
                        // X not 16-byte aligned (a column range starting at an odd
                        // column): the same slice as VW element loads
#pragma unroll
                        for (int q = 0; q < VW; ++q) acc[q] = fma(aa, __ldg(xr + q), acc[q]);
                    }
                } else if (c < kact) {
                    // ragged tail (k not a multiple of VW); lanes past the last column
                    // skip both branches so the warp issues the vector FMAs only once
#pragma unroll
                    for (int q = 0; q < VW; ++q)
                        if (c + q < kact) acc[q] = fma(aa, __ldg(xr + q), acc[q]);
                }
            }
        }
        T *yr = Y + row * ldy + c;
#pragma unroll
        for (int q = 0; q < VW; ++q) {
            if (c + q >= kact) break;
            const T s = alpha * (alpha_col ? (T)alpha_col[c + q] : (T)1);
            yr[q] = beta == (T)0 ? s * acc[q] : s * acc[q] + beta * yr[q];
        }
    }
}

// lanes per row for the vectorised SpMM: the smallest of 4/8/16/32 covering k
template <typename T>
static int spmm_vec_lanes(int k)
{
    const int need = (k + (16 / (int)sizeof(T)) - 1) / (16 / (int)sizeof(T));
    return need <= 4 ? 4 : (need <= 8 ? 8 : (need <= 16 ? 16 : 32));
}

static bool aligned16(const void *p, long ld, size_t es)
{
    return ((uintptr_t)p & 15u) == 0 && ((ld * (long)es) & 15) == 0;
}

// single-column SpMV: a warp splits the row's nonzeros, shuffle reduction
template <typename VT, typename XT, typename AT>
__global__ void __launch_bounds__(256)
k_spmv(int n, const int *__restrict__ rp, const int *__restrict__ ci, const VT *__restrict__ val,
       const XT *__restrict__ X, long ldx, XT *__restrict__ Y, long ldy, AT alpha,
       const double *__restrict__ alpha_col, AT beta, const int *__restrict__ ncols_dev)
{
    const int lane = threadIdx.x & 31;
    const long row = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    if (ncols_dev && *ncols_dev < 1) return;
    AT acc = 0;
    for (int e = rp[row] + lane; e < rp[row + 1]; e += 32)
        acc = fma((AT)__ldg(val + e), (AT)__ldg(X + (long)__ldg(ci + e) * ldx), acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
    if (lane == 0) {
        AT s = alpha * (alpha_col ? (AT)alpha_col[0] : (AT)1);
        Y[row * ldy] = (XT)(beta == (AT)0 ? s * acc : s * acc + beta * (AT)Y[row * ldy]);
    }
}

// FP64 SpMM with a lane shape fitted to k: a group of L lanes (L = 4, 8, 16) owns
// a row and every lane VW consecutive columns (VW = 1..8, element loads), so
// that L VW covers k with few idle lanes -- the FP64 pipe spends its issue slots
// on idle lanes too, and k (the unconverged columns) shrinks during a solve.
// 32 / L rows per warp; (column, value) pairs broadcast by group shuffles. Every
// lane runs the same instruction stream: a lane whose columns run past k reads
// the window [k - VW, k) instead (VW <= k, so it stays inside the range) and
// stores only the columns it owns, so that no lane diverges in the inner loop.
// one row group of the FP64 SpMM below: the L lanes of group `sub` own row `row`
template <int L, int VW>
__device__ __forceinline__ void
spmm64_row(long row, int sl, unsigned gmask, int kact, int k, const int *__restrict__ rp,
           const int *__restrict__ ci, const double *__restrict__ val, const double *__restrict__ X, long ldx,
           double *__restrict__ Y, long ldy, double alpha, const double *__restrict__ alpha_col, double beta)
{
    const int beg = rp[row], end = rp[row + 1];
    for (int c0 = 0; c0 < kact; c0 += L * VW) {
        const int c = c0 + sl * VW;                       // first column this lane owns
        const int cb = min(c, k - VW);                    // first column it reads
        double acc[VW];
#pragma unroll
        for (int q = 0; q < VW; ++q) acc[q] = 0;
        for (int base = beg; base < end; base += L) {
            const int e = base + sl;
            int j = 0;
            double a = 0;
            if (e < end) { j = __ldg(ci + e); a = __ldg(val + e); }
            const int cnt = min(L, end - base);
#pragma unroll 4
            for (int t = 0; t < cnt; ++t) {
                const int jj = __shfl_sync(gmask, j, t, L);
                const double aa = __shfl_sync(gmask, a, t, L);
                const double *xr = X + (long)jj * ldx + cb;
#pragma unroll
                for (int q = 0; q < VW; ++q) acc[q] = fma(aa, __ldg(xr + q), acc[q]);
            }
        }
        double *yr = Y + row * ldy + cb;
#pragma unroll
        for (int q = 0; q < VW; ++q) {
            const int col = cb + q;
            if (col < c || col >= kact) continue;
            const double s = alpha * (alpha_col ? alpha_col[col] : 1.0);
            yr[q] = beta == 0.0 ? s * acc[q] : s * acc[q] + beta * yr[q];
        }
    }
}

template <int L, int VW>
__global__ void __launch_bounds__(256)
k_spmm64_lv(int n, const int *__restrict__ rp, const int *__restrict__ ci, const double *__restrict__ val,
            const double *__restrict__ X, long ldx, double *__restrict__ Y, long ldy, int k, double alpha,
            const double *__restrict__ alpha_col, double beta, const int *__restrict__ ncols_dev)
{
    constexpr int RPW = 32 / L;
    const int lane = threadIdx.x & 31;
    const int sub = lane / L, sl = lane % L;
    const unsigned gmask = (L == 32) ? FULL : (((1u << L) - 1u) << (sub * L));
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long row = warp * RPW + sub;
    int kact = k;
    if (ncols_dev) kact = min(k, *ncols_dev);
    if (row >= n || kact <= 0) return;                    // uniform within the row group
    spmm64_row<L, VW>(row, sl, gmask, kact, k, rp, ci, val, X, ldx, Y, ldy, alpha, alpha_col, beta);
}

// ---------------------------------------------------------------- FP32-pair SpMM
// The FP64 product Y = A X computed on the FP32 pipe, which GB300 issues ~64x
// faster than FP64. Every value is held as an unevaluated sum hi + lo of two
// floats (a 48-bit significand): A once per matrix, scaled by a power of two 2^-s
// so that |a| < 1; X split per call. Each term a x is formed with the error-free
// product of the leading parts (hi*hi exactly as p + e by one FMA, Dekker /
// Kahan's TwoProduct) plus the two cross terms, and summed into a (hi, lo) pair
// per output by Knuth's TwoSum (the pair renormalised after every L terms), so
// the roundings left are the ~2^-48 relative ones of the splits, of the cross
// terms and of the low-order accumulator -- ~1e-14 of sum |a_ij x_j| against
// ~1e-16 for FP64. Results are rebuilt as doubles (exponent shifted back
// by s) with one FP64 add per output. Operations are written with the _rn
// intrinsics so that the compiler does not contract them into FMAs.
// Range: x with |x| >= 2^100 (or non-finite) marks the split, and the product
// then runs the FP64 loop above instead (a device-side switch, uniform per
// launch); |x| < 2^-126 is flushed to zero, |x| < 2^-74 keeps only its leading
// part -- absolute errors below 2^-97 |a| on entries that small.

// (hi, lo) of one double by bit manipulation (no FP64 instruction): hi keeps the
// leading 24 significand bits (truncated), lo the remaining 29 rounded to 24
__device__ __forceinline__ float2 pair_split(double x, int &bad)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7ff);
    const unsigned sign = hi & 0x80000000u;
    if (e >= 1023 + 100) { bad = 1; return make_float2(0.f, 0.f); }
    if (e < 1023 - 126) return make_float2(0.f, 0.f);
    const unsigned hb = sign | ((unsigned)(e - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    float l = 0.f;
    const unsigned rem = lo & 0x1fffffffu;
    if (e >= 949 && rem) l = __fmul_rn(__uint2float_rn(rem), __uint_as_float(sign | ((unsigned)(e - 948) << 23)));
    return make_float2(__uint_as_float(hb), l);
}

// f * 2^s exactly as a double (f normal or zero; subnormal f flushes to zero)
__device__ __forceinline__ double pair_f2d(float f, int s)
{
    const unsigned b = __float_as_uint(f);
    const int e8 = (int)((b >> 23) & 0xff);
    if (e8 == 0) return 0.0;
    const unsigned hi = (b & 0x80000000u) | ((unsigned)(e8 + 896 + s) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)((b & 7u) << 29));
}

// split an n x k block of X (leading dimension ldx) into pairs, leading dimension k:
// blockIdx.y strides the columns in 32s, the x dimension the rows (one row per
// thread-column group, no division)
__global__ void __launch_bounds__(256)
k_pair_split(int n, int k, const double *__restrict__ X, long ldx, float2 *__restrict__ Xs, int *flag, int epoch)
{
    int bad = 0;
    const int lane = threadIdx.x & 31, c = blockIdx.y * 32 + lane;
    const int rstride = gridDim.x * (blockDim.x >> 5);
    if (c < k)
        for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += rstride)
            Xs[(long)r * k + c] = pair_split(X[(long)r * ldx + c], bad);
    if (__any_sync(FULL, bad) && lane == 0) *flag = epoch;
}

// matrix values: max |a| (as ordered bits of a non-negative double), then the split
__global__ void k_pair_absmax(int nnz, const double *__restrict__ v, unsigned long long *meta)
{
    unsigned long long m = 0;
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (long)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v[e]));
        m = b > m ? b : m;
    }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(FULL, m, o);
        m = w > m ? w : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(meta, m);
}

__global__ void k_pair_vals(int nnz, const double *__restrict__ v, float2 *__restrict__ vp, int *meta)
{
    const unsigned long long mb = *(const unsigned long long *)meta;
    // s with max |a| 2^-s in [0.5, 1); s = 0 for an all-zero matrix; non-finite
    // values or |s| > 700 leave s = 4096, which sends every product to the FP64 loop
    int s = 0;
    const int em = (int)((mb >> 52) & 0x7ff);
    if (em == 0x7ff) s = 4096;
    else if (mb) s = em - 1022;
    if (s != 4096 && (s > 700 || s < -700)) s = 4096;
    if (blockIdx.x == 0 && threadIdx.x == 0) meta[2] = s;
    if (s == 4096) return;
    const double sc = ldexp(1.0, -s);
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (long)gridDim.x * blockDim.x) {
        const double a = v[e] * sc;
        const float h = __double2float_rn(a);
        vp[e] = make_float2(h, __double2float_rn(a - (double)h));
    }
}

template <int L, int VW>
__global__ void __launch_bounds__(256)
k_spmm_pair(int n, const int *__restrict__ rp, const int *__restrict__ ci, const float2 *__restrict__ vp,
            const int *__restrict__ meta, const float2 *__restrict__ Xs, const double *__restrict__ val,
            const double *__restrict__ X, long ldx, double *__restrict__ Y, long ldy, int k,
            const int *__restrict__ flag, int epoch)
{
    constexpr int RPW = 32 / L;
    const int lane = threadIdx.x & 31;
    const int sub = lane / L, sl = lane % L;
    const unsigned gmask = (L == 32) ? FULL : (((1u << L) - 1u) << (sub * L));
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long row = warp * RPW + sub;
    if (row >= n) return;                                 // uniform within the row group
    const int s = meta[2];
    if (*flag == epoch || s == 4096) {                    // out of the pair range: FP64
        spmm64_row<L, VW>(row, sl, gmask, k, k, rp, ci, val, X, ldx, Y, ldy, 1.0, nullptr, 0.0);
        return;
    }
    const int beg = rp[row], end = rp[row + 1];
    for (int c0 = 0; c0 < k; c0 += L * VW) {
        const int c = c0 + sl * VW;
        const int cb = min(c, k - VW);
        float sh[VW], sw[VW];
#pragma unroll
        for (int q = 0; q < VW; ++q) { sh[q] = 0.f; sw[q] = 0.f; }
        for (int base = beg; base < end; base += L) {
            const int e = base + sl;
            int j = 0;
            float2 a = make_float2(0.f, 0.f);
            if (e < end) { j = __ldg(ci + e); a = __ldg(vp + e); }
            const int cnt = min(L, end - base);
#pragma unroll 2
            for (int t = 0; t < cnt; ++t) {
                const int jj = __shfl_sync(gmask, j, t, L);
                const float ah = __shfl_sync(gmask, a.x, t, L);
                const float al = __shfl_sync(gmask, a.y, t, L);
                const float2 *xr = Xs + (long)jj * k + cb;
#pragma unroll
                for (int q = 0; q < VW; ++q) {
                    const float2 x = __ldg(xr + q);
                    const float p = __fmul_rn(ah, x.x);
                    float er = fmaf(ah, x.x, -p);                 // ah xh - p, exact
                    er = fmaf(ah, x.y, er);
                    er = fmaf(al, x.x, er);
                    const float t1 = __fadd_rn(sh[q], p);           // TwoSum(sh, p)
                    const float z = __fsub_rn(t1, sh[q]);
                    const float d = __fadd_rn(__fsub_rn(sh[q], __fsub_rn(t1, z)), __fsub_rn(p, z));
                    sh[q] = t1;
                    sw[q] = __fadd_rn(sw[q], __fadd_rn(d, er));
                }
            }
            // renormalise after every L terms (FastTwoSum): |sw| stays near ulp(sh)
#pragma unroll
            for (int q = 0; q < VW; ++q) {
                const float s2 = __fadd_rn(sh[q], sw[q]);
                sw[q] = __fsub_rn(sw[q], __fsub_rn(s2, sh[q]));
                sh[q] = s2;
            }
        }
        double *yr = Y + row * ldy + cb;
#pragma unroll
        for (int q = 0; q < VW; ++q) {
            const int col = cb + q;
            if (col < c || col >= k) continue;
            yr[q] = pair_f2d(sh[q], s) + pair_f2d(sw[q], s);
        }
    }
}

// (L, VW) with the fewest idle lane slots for k columns (ties: the larger L)
static void spmm64_shape(int k, int *Lo, int *VWo)
{
    double best = -1;
    for (int L = 16; L >= 4; L >>= 1) {
        int vw = (k + L - 1) / L;
        if (vw > 8) vw = 8;
        const int cols = L * vw, chunks = (k + cols - 1) / cols;
        const double eff = (double)k / ((double)chunks * cols);
        if (eff > best + 1e-12) {
            best = eff;
            *Lo = L;
            *VWo = vw;
        }
    }
}

#define SPMM64_CASE(LL, VV)                                                                               \
    if (L == LL && VW == VV) {                                                                            \
        GB_LAUNCH(ctx, (k_spmm64_lv<LL, VV>), grid, 256, 0, A->n, A->rp, A->ci, A->v, X, ldx, Y, ldy, k, alpha, \
                  alpha_col, beta, ncols_dev);                                                            \
        return GCGE_GPU_OK;                                                                               \
    }
#define SPMM64_L(LL) SPMM64_CASE(LL, 1) SPMM64_CASE(LL, 2) SPMM64_CASE(LL, 3) SPMM64_CASE(LL, 4) \
    SPMM64_CASE(LL, 5) SPMM64_CASE(LL, 6) SPMM64_CASE(LL, 7) SPMM64_CASE(LL, 8)

static int spmm64_lv_launch(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const double *X, long ldx, double *Y,
                            long ldy, int k, double alpha, const double *alpha_col, double beta,
                            const int *ncols_dev)
{
    int L = 16, VW = 4;
    spmm64_shape(k, &L, &VW);
    const long warps = ((long)A->n * L + 31) / 32;
    const int grid = ceil_div_l(warps * 32, 256);
    SPMM64_L(4)
    SPMM64_L(8)
    SPMM64_L(16)
    return gb_fail(ctx, GCGE_GPU_ERR_ARG);
}

// ---- FP32-pair path: per-matrix pairs (lazy), per-call split of X
static int pair_mat(gcge_gpu_ctx *ctx, const gcge_gpu_mat *Ac)
{
    gcge_gpu_mat *A = (gcge_gpu_mat *)Ac;
    if (A->vpair) return GCGE_GPU_OK;
    const size_t nz = A->nnz > 0 ? (size_t)A->nnz : 1;
    if (cudaMalloc(&A->vpair, sizeof(float2) * nz) != cudaSuccess) {
        A->vpair = nullptr;
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    if (cudaMalloc(&A->pair_meta, 4 * sizeof(int)) != cudaSuccess) {
        cudaFree(A->vpair);
        A->vpair = nullptr;
        A->pair_meta = nullptr;
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    if (cudaMemsetAsync(A->pair_meta, 0, 4 * sizeof(int), ctx->stream) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    const int grid = ctx->num_sms * 8;
    GB_LAUNCH(ctx, k_pair_absmax, grid, 256, 0, A->nnz, A->v, (unsigned long long *)A->pair_meta);
    GB_LAUNCH(ctx, k_pair_vals, grid, 256, 0, A->nnz, A->v, (float2 *)A->vpair, A->pair_meta);
    return GCGE_GPU_OK;
}

static int pair_split_x(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx)
{
    const size_t need = (size_t)2 * n * k;
    if (ctx->pairbuf_cap < need) {
        if (ctx->pairbuf) {
            if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
            cudaFree(ctx->pairbuf);
            ctx->pairbuf = nullptr;
            ctx->pairbuf_cap = 0;
        }
        if (cudaMalloc(&ctx->pairbuf, need * sizeof(float)) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
        ctx->pairbuf_cap = need;
    }
    ctx->pair_epoch = ctx->pair_epoch == 0x7fffffff ? 1 : ctx->pair_epoch + 1;
    GB_PROF(ctx, GB_K_BLAS1, 16.0 * n * k, 0.0);
    const int ct = (k + 31) / 32;
    const int gx = ceil_div_l((long)ctx->num_sms * 16, ct) < ceil_div_l(n, 8) ? ceil_div_l((long)ctx->num_sms * 16, ct)
                                                                                : ceil_div_l(n, 8);
    GB_LAUNCH(ctx, k_pair_split, dim3(gx, ct), 256, 0, n, k, X, ldx, (float2 *)ctx->pairbuf, ctx->dev_pairflag,
              ctx->pair_epoch);
    return GCGE_GPU_OK;
}

#define SPMMP_CASE(LL, VV)                                                                                    \
    if (L == LL && VW == VV) {                                                                                \
        GB_LAUNCH(ctx, (k_spmm_pair<LL, VV>), grid, 256, 0, A->n, A->rp, A->ci, (const float2 *)A->vpair,      \
                  A->pair_meta, (const float2 *)ctx->pairbuf, A->v, X, ldx, Y, ldy, k, ctx->dev_pairflag,       \
                  ctx->pair_epoch);                                                                           \
        return GCGE_GPU_OK;                                                                                   \
    }
#define SPMMP_L(LL) SPMMP_CASE(LL, 1) SPMMP_CASE(LL, 2) SPMMP_CASE(LL, 3) SPMMP_CASE(LL, 4) \
    SPMMP_CASE(LL, 5) SPMMP_CASE(LL, 6) SPMMP_CASE(LL, 7)

// Lane shape of the pair product: the fewest idle lane slots (as for FP64);
// among equals two columns per lane first, then the larger L. Measured on the Q1
// cube 96^3 stiffness (us per product): k = 16: (8, 2) 355, (4, 4) 387, (16, 1)
// 459; k = 32: (16, 2) 592, (8, 4) 640, (4, 8) 1101; k = 56: (8, 7) 852;
// k = 64: (16, 4) 1244, (8, 8) 2140 -- eight contiguous columns per lane is a
// slow gather pattern, so VW stops at 7.
static void spmm_pair_shape(int k, int *Lo, int *VWo)
{
    double best = -1;
    for (int L = 16; L >= 4; L >>= 1) {
        int vw = (k + L - 1) / L;
        if (vw > 7) vw = 7;
        const int cols = L * vw, chunks = (k + cols - 1) / cols;
        const double eff = (double)k / ((double)chunks * cols);
        if (eff > best + 1e-12 || (eff > best - 1e-12 && vw == 2 && *VWo != 2)) {
            best = eff > best ? eff : best;
            *Lo = L;
            *VWo = vw;
        }
    }
}

// Y = A X from the split left in ctx->pairbuf by pair_split_x
static int spmm_pair_launch(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const double *X, long ldx, double *Y,
                            long ldy, int k)
{
    int st = pair_mat(ctx, A);
    if (st) return st;
    ctx->spmm_launches++;
    GB_PROF(ctx, GB_K_SPMMPAIR, 12.0 * A->nnz + 4.0 * (A->n + 1) + 16.0 * A->n * k, 2.0 * A->nnz * k);
    int L = 16, VW = 0;
    spmm_pair_shape(k, &L, &VW);
    const long warps = ((long)A->n * L + 31) / 32;
    const int grid = ceil_div_l(warps * 32, 256);
    SPMMP_L(4)
    SPMMP_L(8)
    SPMMP_L(16)
    return gb_fail(ctx, GCGE_GPU_ERR_ARG);
}

// the products this path takes: two or more columns, Y = A X
static bool pair_applies(const gcge_gpu_ctx *ctx, int k, double alpha, const double *alpha_col, double beta,
                         const int *ncols_dev)
{
    return ctx->spmm_pair && k >= 2 && !alpha_col && beta == 0.0 && !ncols_dev && alpha == 1.0;
}

extern "C" int gb_spmm_ab(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, const double *X,
                          long ldx, double *YA, double *YB, long ldy, int k)
{
    if (k <= 0 || A->n <= 0) return GCGE_GPU_OK;
    if (!pair_applies(ctx, k, 1.0, nullptr, 0.0, nullptr)) {
        int st = gb_spmm(ctx, A, X, ldx, YA, ldy, k, 1.0, nullptr, 0.0, nullptr);
        if (!st && B) st = gb_spmm(ctx, B, X, ldx, YB, ldy, k, 1.0, nullptr, 0.0, nullptr);
        return st;
    }
    int st = pair_split_x(ctx, A->n, k, X, ldx);
    if (!st) st = spmm_pair_launch(ctx, A, X, ldx, YA, ldy, k);
    if (!st && B) st = spmm_pair_launch(ctx, B, X, ldx, YB, ldy, k);
    return st;
}

extern "C" int gb_spmm(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const double *X, long ldx, double *Y,
                       long ldy, int k, double alpha, const double *alpha_col, double beta,
                       const int *ncols_dev)
{
    if (k <= 0 || A->n <= 0) return GCGE_GPU_OK;
    if (pair_applies(ctx, k, alpha, alpha_col, beta, ncols_dev)) {
        int st = pair_split_x(ctx, A->n, k, X, ldx);
        return st ? st : spmm_pair_launch(ctx, A, X, ldx, Y, ldy, k);
    }
    ctx->spmm_launches++;
    GB_PROF(ctx, GB_K_SPMM64, 12.0 * A->nnz + 4.0 * (A->n + 1) + (beta != 0.0 ? 24.0 : 16.0) * A->n * k,
            2.0 * A->nnz * k);
    // one column: matrices whose longest row is short (stencils, meshes) take a
    // thread per row -- a warp-wide reduction per row would cost five FP64 adds on
    // every lane, and the FP64 pipe is the narrow one; long rows keep a warp per row
    if (k == 1) {
        if (A->max_row_nnz <= 64.0) {
            const int grid = ceil_div_l((long)A->n, 256);
            GB_LAUNCH(ctx, (k_spmm64_lv<1, 1>), grid, 256, 0, A->n, A->rp, A->ci, A->v, X, ldx, Y, ldy, 1, alpha,
                      alpha_col, beta, ncols_dev);
            return GCGE_GPU_OK;
        }
        int grid = ceil_div_l((long)A->n * 32, 256);
        GB_LAUNCH(ctx, (k_spmv<double, double, double>), grid, 256, 0, A->n, A->rp, A->ci, A->v, X, ldx,
                  Y, ldy, alpha, alpha_col, beta, ncols_dev);
        return GCGE_GPU_OK;
    }
    return spmm64_lv_launch(ctx, A, X, ldx, Y, ldy, k, alpha, alpha_col, beta, ncols_dev);
}

extern "C" int gb_spmm32(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const float *X, long ldx, float *Y,
                         long ldy, int k, const int *ncols_dev)
{
    if (k <= 0 || A->n <= 0) return GCGE_GPU_OK;
    if (!A->v32) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    ctx->spmm_launches++;
    GB_PROF(ctx, GB_K_SPMM32, 8.0 * A->nnz + 4.0 * (A->n + 1) + 8.0 * A->n * k, 2.0 * A->nnz * k);
    if (k == 1) {
        int grid = ceil_div_l((long)A->n * 32, 256);
        GB_LAUNCH(ctx, (k_spmv<float, float, float>), grid, 256, 0, A->n, A->rp, A->ci, A->v32, X, ldx,
                  Y, ldy, 1.0f, (const double *)nullptr, 0.0f, ncols_dev);
    } else {
        if (aligned16(X, ldx, sizeof(float)) && aligned16(Y, ldy, sizeof(float))) {
            const int L = spmm_vec_lanes<float>(k);
            const long warps = ((long)A->n * L + 31) / 32;
            const int grid = ceil_div_l(warps * 32, 256);
            if (L == 4)
                GB_LAUNCH(ctx, (k_spmm_vec<float, 4>), grid, 256, 0, A->n, A->rp, A->ci, A->v32, X, ldx, Y, ldy, k,
                          1.0f, (const double *)nullptr, 0.0f, ncols_dev);
            else if (L == 8)
                GB_LAUNCH(ctx, (k_spmm_vec<float, 8>), grid, 256, 0, A->n, A->rp, A->ci, A->v32, X, ldx, Y, ldy, k,
                          1.0f, (const double *)nullptr, 0.0f, ncols_dev);
            else if (L == 16)
                GB_LAUNCH(ctx, (k_spmm_vec<float, 16>), grid, 256, 0, A->n, A->rp, A->ci, A->v32, X, ldx, Y, ldy, k,
                          1.0f, (const double *)nullptr, 0.0f, ncols_dev);
            else
                GB_LAUNCH(ctx, (k_spmm_vec<float, 32>), grid, 256, 0, A->n, A->rp, A->ci, A->v32, X, ldx, Y, ldy, k,
                          1.0f, (const double *)nullptr, 0.0f, ncols_dev);
        } else {
            long warps = (long)A->n * ((k + 63) / 64);
            int grid = ceil_div_l(warps * 32, 256);
            GB_LAUNCH(ctx, (k_spmm<float, float, float>), grid, 256, 0, A->n, A->rp, A->ci, A->v32, X, ldx, Y,
                      ldy, k, 1.0f, (const double *)nullptr, 0.0f, ncols_dev);
        }
    }
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- AXPBY
// warp-per-row loop over an n x k block: lanes walk the columns of one row
#define ROWS_BY_WARP(n, r)                                                             \
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < (n);         \
         r += ((long)gridDim.x * blockDim.x) >> 5)

__global__ void k_axpby(int n, int k, double a, const double *__restrict__ X, long ldx, double b,
                        double *__restrict__ Y, long ldy)
{
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) {
        double *y = Y + r * ldy + c;
        if (a == 0.0) *y = b * *y;
        else if (b == 0.0) *y = (a == 1.0) ? X[r * ldx + c] : a * X[r * ldx + c];
        else *y = a * X[r * ldx + c] + b * *y;
    }
}

// blocks of 8 warps for a warp-per-row loop, capped at 16 blocks per SM
static int row_grid(gcge_gpu_ctx *ctx, long rows)
{
    long g = (rows + 7) / 8, cap = (long)ctx->num_sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

static int elem_grid(gcge_gpu_ctx *ctx, long total)
{
    long g = (total + 255) / 256;
    long cap = (long)ctx->num_sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

extern "C" int gb_axpby(gcge_gpu_ctx *ctx, int n, int k, double a, const double *X, long ldx, double b,
                        double *Y, long ldy)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    GB_PROF(ctx, GB_K_BLAS1, (a == 0.0 || b == 0.0 ? 16.0 : 24.0) * n * k, 2.0 * n * k);
    GB_LAUNCH(ctx, k_axpby, row_grid(ctx, n), 256, 0, n, k, a, X, ldx, b, Y, ldy);
    return GCGE_GPU_OK;
}

// per-column source index and scale of a gather, staged once per block in
// shared memory (scale 1, or 1 / lambda of the column when |lambda| > 1)
__device__ __forceinline__ void gather_setup(int k, const int *idx, const double *eval, int mode, int *si,
                                             double *ss)
{
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        const int src = idx ? idx[c] : c;
        si[c] = src;
        double s = 1.0;
        if (mode == 1) {
            const double l = eval[src];
            s = fabs(l) <= 1.0 ? 1.0 : 1.0 / l;
        }
        ss[c] = s;
    }
    __syncthreads();
}

__global__ void k_gather_cols(int n, int k, const double *__restrict__ X, long ldx, const int *__restrict__ idx,
                              double *__restrict__ Y, long ldy, const double *__restrict__ eval, int mode)
{
    extern __shared__ double gsm[];
    double *ss = gsm;
    int *si = (int *)(gsm + k);
    gather_setup(k, idx, eval, mode, si, ss);
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) {
        const double s = ss[c];
        const double x = X[r * ldx + si[c]];
        Y[r * ldy + c] = s != 1.0 ? s * x : x;
    }
}

extern "C" int gb_gather_cols(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const int *idx_dev,
                              double *Y, long ldy, const double *eval_dev, int mode)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    if (k > 4096) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    GB_LAUNCH(ctx, k_gather_cols, row_grid(ctx, n), 256, (size_t)k * 12, n, k, X, ldx, idx_dev, Y, ldy,
              eval_dev, mode);
    return GCGE_GPU_OK;
}

// initial residual of the correction equation from products already formed:
// R[:, c] = s_c (lam_c BX[:, bi[c]] - AX[:, ai[c]]) with the scale of the initial
// guess, s_c = 1 if |lam_c| <= 1 else 1 / lam_c
__global__ void k_w_residual(int n, int k, const double *__restrict__ AX, long ldax, const int *__restrict__ ai,
                             const double *__restrict__ BX, long ldbx, const int *__restrict__ bi,
                             const double *__restrict__ lam, double *__restrict__ R, long ldr)
{
    extern __shared__ double gsm[];
    double *ss = gsm;
    int *si = (int *)(gsm + k);
    gather_setup(k, nullptr, lam, 1, si, ss);
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) {
        const double v = lam[c] * BX[r * ldbx + bi[c]] - AX[r * ldax + ai[c]];
        R[r * ldr + c] = ss[c] != 1.0 ? ss[c] * v : v;
    }
}

extern "C" int gb_w_residual(gcge_gpu_ctx *ctx, int n, int k, const double *AX, long ldax, const int *ai,
                             const double *BX, long ldbx, const int *bi, const double *lam, double *R, long ldr)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    if (k > 4096) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    GB_PROF(ctx, GB_K_BLAS1, 24.0 * n * k, 3.0 * n * k);
    GB_LAUNCH(ctx, k_w_residual, row_grid(ctx, n), 256, (size_t)k * 12, n, k, AX, ldax, ai, BX, ldbx, bi, lam, R,
              ldr);
    return GCGE_GPU_OK;
}

__global__ void k_fill_random(int n, int k, double *X, long ldx, int col0, unsigned long long seed)
{
    const long total = (long)n * k;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long r = t / k;
        const int c = (int)(t - r * k);
        unsigned long long z = seed ^ ((unsigned long long)((long)(col0 + c) * n + r) * 0xD1B54A32D192ED03ULL);
        z += 0x9E3779B97F4A7C15ULL;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z ^= z >> 31;
        X[r * ldx + c] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
}

extern "C" int gb_fill_random(gcge_gpu_ctx *ctx, int n, int k, double *X, long ldx, int col0,
                              unsigned long long seed)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_fill_random, elem_grid(ctx, (long)n * k), 256, 0, n, k, X, ldx, col0, seed);
    return GCGE_GPU_OK;
}

__global__ void k_d2f(int n, int k, const double *__restrict__ X, long ldx, float *__restrict__ Y, long ldy)
{
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) Y[r * ldy + c] = (float)X[r * ldx + c];
}
__global__ void k_f2d(int n, int k, const float *__restrict__ X, long ldx, double *__restrict__ Y, long ldy)
{
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) Y[r * ldy + c] = (double)X[r * ldx + c];
}
extern "C" int gb_convert_d2f(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, float *Y, long ldy)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_d2f, row_grid(ctx, n), 256, 0, n, k, X, ldx, Y, ldy);
    return GCGE_GPU_OK;
}
extern "C" int gb_convert_f2d(gcge_gpu_ctx *ctx, int n, int k, const float *X, long ldx, double *Y, long ldy)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_f2d, row_grid(ctx, n), 256, 0, n, k, X, ldx, Y, ldy);
    return GCGE_GPU_OK;
}

// Dirichlet rows (app/csr/gcge_app_csr.c:130-183): B row has no |b| > 1e-20 and
// the A row exactly one |a| > 1e-20 -> zero that row of X.
__global__ void k_dirichlet(int n, const int *arp, const double *av, const int *brp, const double *bv, int k,
                            double *X, long ldx)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool zero_b = true;
        for (int j = brp[i]; j < brp[i + 1]; ++j)
            if (fabs(bv[j]) > 1e-20) { zero_b = false; break; }
        if (!zero_b) continue;
        int cnt = 0;
        for (int j = arp[i]; j < arp[i + 1]; ++j)
            if (fabs(av[j]) > 1e-20) cnt++;
        if (cnt == 1)
            for (int c = 0; c < k; ++c) X[(long)i * ldx + c] = 0.0;
    }
}
extern "C" int gb_dirichlet_zero(gcge_gpu_ctx *ctx, const gcge_gpu_mat *A, const gcge_gpu_mat *B, int k,
                                 double *X, long ldx)
{
    if (!A || !B || k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_dirichlet, elem_grid(ctx, A->n), 256, 0, A->n, A->rp, A->v, B->rp, B->v, k, X, ldx);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- per-column reductions
// Stage 1: block b covers rows [b*R, (b+1)*R) (R fixed by n), 32-column slab per
// blockIdx.y; partial[b * k + c]. Stage 2: fixed-order sum over b.
#define RED_ROWS 1024
template <int MODE>
__global__ void __launch_bounds__(256)
k_coldot_partial(int n, int k, const double *__restrict__ X, long ldx, const double *__restrict__ Y, long ldy,
                 const double *__restrict__ Z, long ldz, const double *__restrict__ eval,
                 const int *__restrict__ idx, double *__restrict__ part, int bnorm = 0)
{
    // MODE 0: sum X*Y. MODE 1: residual triple (sum (Y - l Z)^2, sum X^2, sum Z^2), Z may be NULL (= X);
    // bnorm != 0 ("BR": only the residual and the B-norm are used) skips X (when Z is given) and sum X^2
    // (reported as sum Z^2): three FP64 operations per entry instead of four, the FP64 pipe being the
    // limit of this pass on GB300
    __shared__ double sh[3][8][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int c = blockIdx.y * 32 + tx;
    const long r0 = (long)blockIdx.x * RED_ROWS;
    const long r1 = min((long)n, r0 + RED_ROWS);
    double s0 = 0, s1 = 0, s2 = 0;
    if (c < k) {
        double l = 0;
        if (MODE == 1) l = eval[idx ? idx[c] : c];
        for (long r = r0 + ty; r < r1; r += 8) {
            if (MODE == 0) {
                s0 = fma(X[r * ldx + c], Y[r * ldy + c], s0);
            } else if (bnorm) {
                const double bx = Z ? Z[r * ldz + c] : X[r * ldx + c];
                const double res = Y[r * ldy + c] - l * bx;
                s0 = fma(res, res, s0);
                s2 = fma(bx, bx, s2);
            } else {
                const double x = X[r * ldx + c];
                const double bx = Z ? Z[r * ldz + c] : x;
                const double res = Y[r * ldy + c] - l * bx;
                s0 = fma(res, res, s0);
                s1 = fma(x, x, s1);
            }
        }
    }
    sh[0][ty][tx] = s0;
    sh[1][ty][tx] = s1;
    sh[2][ty][tx] = s2;
    __syncthreads();
    if (ty == 0 && c < k) {
        double t0 = 0, t1 = 0, t2 = 0;
        for (int q = 0; q < 8; ++q) { t0 += sh[0][q][tx]; t1 += sh[1][q][tx]; t2 += sh[2][q][tx]; }
        if (MODE == 1) {
            if (bnorm) t1 = t2;                       // only the B-norm was formed
            else t2 = t1;                             // only the 2-norm was formed
        }
        const int w = MODE == 0 ? 1 : 3;
        double *p = part + ((long)blockIdx.x * k + c) * w;
        p[0] = t0;
        if (MODE == 1) { p[1] = t1; p[2] = t2; }
    }
}

__global__ void k_sum_partials(int nblk, int width, const double *__restrict__ part, double *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= width) return;
    double s = 0;
    for (int b = 0; b < nblk; ++b) s += part[(long)b * width + c];
    out[c] = s;
}

extern "C" int gb_col_dots(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const double *Y,
                           long ldy, double *out_dev)
{
    if (k <= 0) return GCGE_GPU_OK;
    const int nblk = ceil_div_l(n > 0 ? n : 1, RED_ROWS);
    int st = gb_scratch(ctx, (size_t)nblk * k);
    if (st) return st;
    dim3 grid(nblk, (k + 31) / 32);
    GB_PROF(ctx, GB_K_REDUCE, 16.0 * n * k, 2.0 * n * k);
    GB_LAUNCH(ctx, k_coldot_partial<0>, grid, 256, 0, n, k, X, ldx, Y, ldy, (const double *)nullptr, 0L,
              (const double *)nullptr, (const int *)nullptr, ctx->scratch);
    GB_LAUNCH(ctx, k_sum_partials, (k + 127) / 128, 128, 0, nblk, k, ctx->scratch, out_dev);
    return GCGE_GPU_OK;
}

extern "C" int gb_residual_norms(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const double *AX,
                                 long ldax, const double *BX, long ldbx, const double *eval_dev,
                                 const int *idx_dev, double *out_dev, int bnorm)
{
    if (k <= 0) return GCGE_GPU_OK;
    const int nblk = ceil_div_l(n > 0 ? n : 1, RED_ROWS);
    int st = gb_scratch(ctx, (size_t)nblk * k * 3);
    if (st) return st;
    dim3 grid(nblk, (k + 31) / 32);
    GB_PROF(ctx, GB_K_REDUCE, (BX && !bnorm ? 24.0 : 16.0) * n * k, 6.0 * n * k);
    GB_LAUNCH(ctx, k_coldot_partial<1>, grid, 256, 0, n, k, X, ldx, AX, ldax, BX, ldbx, eval_dev, idx_dev,
              ctx->scratch, bnorm);
    GB_LAUNCH(ctx, k_sum_partials, (3 * k + 127) / 128, 128, 0, nblk, 3 * k, ctx->scratch, out_dev);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- Gram V^T W
// grid (tiles_i, tiles_j, splits); 32x32 output tile, each thread 2x2 outputs;
// 32-row slabs of V and W staged in shared memory.
__global__ void __launch_bounds__(256)
k_gram_partial(int n, int k1, int k2, const double *__restrict__ V, long ldv, const double *__restrict__ W,
               long ldw, double *__restrict__ part, long rows_per_split, int sym)
{
    const int ti = blockIdx.x, tj = blockIdx.y, split = blockIdx.z;
    if (sym && ti > tj) return;
    const int i0 = ti * 32, j0 = tj * 32;
    const long rb = (long)split * rows_per_split;
    const long re = min((long)n, rb + rows_per_split);
    __shared__ double Vs[32][33];
    __shared__ double Ws[32][33];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double a00 = 0, a01 = 0, a10 = 0, a11 = 0;
    for (long r0 = rb; r0 < re; r0 += 32) {
        for (int e = threadIdx.x; e < 1024; e += 256) {
            const int rr = e >> 5, cc = e & 31;
            const long r = r0 + rr;
            Vs[rr][cc] = (r < re && i0 + cc < k1) ? V[r * ldv + i0 + cc] : 0.0;
            Ws[rr][cc] = (r < re && j0 + cc < k2) ? W[r * ldw + j0 + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < 32; ++rr) {
            const double v0 = Vs[rr][2 * ty], v1 = Vs[rr][2 * ty + 1];
            const double w0 = Ws[rr][2 * tx], w1 = Ws[rr][2 * tx + 1];
            a00 = fma(v0, w0, a00);
            a01 = fma(v0, w1, a01);
            a10 = fma(v1, w0, a10);
            a11 = fma(v1, w1, a11);
        }
        __syncthreads();
    }
    double *p = part + (long)split * k1 * k2;
    const int i = i0 + 2 * ty, j = j0 + 2 * tx;
    if (i < k1 && j < k2) p[i + (long)j * k1] = a00;
    if (i < k1 && j + 1 < k2) p[i + (long)(j + 1) * k1] = a01;
    if (i + 1 < k1 && j < k2) p[i + 1 + (long)j * k1] = a10;
    if (i + 1 < k1 && j + 1 < k2) p[i + 1 + (long)(j + 1) * k1] = a11;
}

__global__ void k_gram_reduce(int k1, int k2, int nsplit, const double *__restrict__ part, double *a, int lda,
                              int sym)
{
    const long total = (long)k1 * k2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % k1), j = (int)(t / k1);
        if (sym && i > j) continue;
        double s = 0;
        for (int q = 0; q < nsplit; ++q) s += part[(long)q * total + t];
        a[i + (long)j * lda] = s;
        if (sym && i != j) a[j + (long)i * lda] = s;
    }
}

extern "C" int gb_gram(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *V, long ldv, const double *W,
                       long ldw, double *a_dev, int lda, int sym)
{
    if (k1 <= 0 || k2 <= 0) return GCGE_GPU_OK;
    if (ctx->tc) {
        int st = gb_iscratch(ctx, (size_t)k1 + k2);
        if (st) return st;
        return gb_gram_tc(ctx, n, k1, k2, V, ldv, W, ldw, a_dev, lda, sym, ctx->iscratch);
    }
    const int ti = (k1 + 31) / 32, tj = (k2 + 31) / 32;
    int tiles = sym ? ti * (ti + 1) / 2 : ti * tj;
    if (tiles < 1) tiles = 1;
    long target = (long)ctx->num_sms * 4;
    long nsplit = target / tiles;
    long max_split = (n + 255) / 256;
    if (nsplit > max_split) nsplit = max_split;
    if (nsplit < 1) nsplit = 1;
    long rps = ((n + nsplit - 1) / nsplit + 31) / 32 * 32;
    if (rps < 32) rps = 32;
    nsplit = (n + rps - 1) / rps;
    if (nsplit < 1) nsplit = 1;
    int st = gb_scratch(ctx, (size_t)nsplit * k1 * k2);
    if (st) return st;
    dim3 grid(ti, tj, (unsigned)nsplit);
    GB_PROF(ctx, GB_K_GRAM, 8.0 * n * (k1 + k2), sym ? 1.0 * n * k1 * (k1 + 1) : 2.0 * n * k1 * k2);
    GB_LAUNCH(ctx, k_gram_partial, grid, 256, 0, n, k1, k2, V, ldv, W, ldw, ctx->scratch, rps, sym);
    GB_LAUNCH(ctx, k_gram_reduce, elem_grid(ctx, (long)k1 * k2), 256, 0, k1, k2, (int)nsplit, ctx->scratch,
              a_dev, lda, sym);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- linear combination X*C
// Y[r, j] = alpha * sum_i X[r, i] C[i + j*ldc] + beta * Y[r, j]; tile 64 rows x 32 cols.
__global__ void __launch_bounds__(256)
k_lincomb(int n, int k1, int k2, const double *__restrict__ X, long ldx, const double *__restrict__ C, int ldc,
          double alpha, double beta, double *__restrict__ Y, long ldy, int upper)
{
    __shared__ double Xs[64][33];
    __shared__ double Cs[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long r0 = (long)blockIdx.x * 64;
    const int j0 = blockIdx.y * 32;
    const int j = j0 + tx;
    double acc[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) acc[q] = 0.0;
    int iend = k1;
    if (upper) iend = min(k1, j0 + 32);
    for (int i0 = 0; i0 < iend; i0 += 32) {
        for (int e = threadIdx.x; e < 64 * 32; e += 256) {
            const int rr = e >> 5, cc = e & 31;
            const long r = r0 + rr;
            Xs[rr][cc] = (r < n && i0 + cc < k1) ? X[r * ldx + i0 + cc] : 0.0;
        }
        for (int e = threadIdx.x; e < 32 * 32; e += 256) {
            const int ii = e & 31, cc = e >> 5;
            Cs[ii][cc] = (i0 + ii < k1 && j0 + cc < k2) ? C[(i0 + ii) + (long)(j0 + cc) * ldc] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int ii = 0; ii < 32; ++ii) {
            const double c = Cs[ii][tx];
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[q] = fma(Xs[ty + 8 * q][ii], c, acc[q]);
        }
        __syncthreads();
    }
    if (j < k2) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const long r = r0 + ty + 8 * q;
            if (r < n) {
                double *y = Y + r * ldy + j;
                *y = beta == 0.0 ? alpha * acc[q] : alpha * acc[q] + beta * *y;
            }
        }
    }
}

extern "C" int gb_lincomb_inplace_ok(const gcge_gpu_ctx *ctx, int k1, int k2)
{
    return ctx->tc && gb_lincomb_tc_inplace_ok(k1, k2);
}

extern "C" int gb_lincomb(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *X, long ldx,
                          const double *C_dev, int ldc, double alpha, double beta, double *Y, long ldy,
                          int upper)
{
    if (n <= 0 || k2 <= 0) return GCGE_GPU_OK;
    if (k1 <= 0) return gb_axpby(ctx, n, k2, 0.0, Y, ldy, beta, Y, ldy);
    if (ctx->tc && gb_lincomb_tc_ok(k1)) return gb_lincomb_tc(ctx, n, k1, k2, X, ldx, C_dev, ldc, alpha, beta, Y, ldy, upper);
    dim3 grid(ceil_div_l(n, 64), (k2 + 31) / 32);
    GB_PROF(ctx, GB_K_LINCOMB, 8.0 * n * k1 + (beta != 0.0 ? 16.0 : 8.0) * n * k2,
            upper ? 1.0 * n * k1 * (k2 + 1) : 2.0 * n * k1 * k2);
    GB_LAUNCH(ctx, k_lincomb, grid, 256, 0, n, k1, k2, X, ldx, C_dev, ldc, alpha, beta, Y, ldy, upper);
    return GCGE_GPU_OK;
}

// Frobenius norm of a small column-major block (one block, fixed order)
__global__ void k_frobenius(int m, int n, const double *a, int lda, double *out)
{
    __shared__ double sh[256];
    double s = 0;
    for (long t = threadIdx.x; t < (long)m * n; t += 256) {
        const double v = a[(t % m) + (t / m) * lda];
        s = fma(v, v, s);
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sqrt(sh[0]);
}
extern "C" int gb_frobenius(gcge_gpu_ctx *ctx, int m, int n, const double *a, int lda, double *out_dev)
{
    GB_LAUNCH(ctx, k_frobenius, 1, 256, 0, m, n, a, lda, out_dev);
    return GCGE_GPU_OK;
}

// out[c] = src[idx[c]] (eigenvalues of the unlocked columns)
__global__ void k_select(int k, const double *src, const int *idx, double *out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < k) out[c] = src[idx[c]];
}
extern "C" int gb_select(gcge_gpu_ctx *ctx, int k, const double *src, const int *idx, double *out)
{
    if (k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_select, (k + 127) / 128, 128, 0, k, src, idx, out);
    return GCGE_GPU_OK;
}

// Y[:, c] = s[c] * X[:, c]
__global__ void k_scale_cols(int n, int k, const double *__restrict__ X, long ldx, const double *__restrict__ s,
                             double *Y, long ldy)
{
    const int lane = threadIdx.x & 31;
    ROWS_BY_WARP(n, r)
    for (int c = lane; c < k; c += 32) Y[r * ldy + c] = s[c] * X[r * ldx + c];
}
extern "C" int gb_scale_cols(gcge_gpu_ctx *ctx, int n, int k, const double *X, long ldx, const double *s, double *Y,
                             long ldy)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    GB_LAUNCH(ctx, k_scale_cols, row_grid(ctx, n), 256, 0, n, k, X, ldx, s, Y, ldy);
    return GCGE_GPU_OK;
}

// Gram V^T W with caller-provided partial-sum storage and stream (no context,
// no allocation): the launcher behind the allocation-free entry point. part
// must hold part_cap doubles; returns GCGE_GPU_ERR_ARG when k1*k2 does not fit
// at least one row split.
extern "C" int gb_gram_fixed_scratch(cudaStream_t stream, int num_sms, int n, int k1, int k2, const double *V,
                                     long ldv, const double *W, long ldw, double *a_dev, int lda, int sym,
                                     double *part, size_t part_cap)
{
    const int ti = (k1 + 31) / 32, tj = (k2 + 31) / 32;
    int tiles = sym ? ti * (ti + 1) / 2 : ti * tj;
    if (tiles < 1) tiles = 1;
    long nsplit = ((long)num_sms * 4) / tiles;
    const long max_split = (n + 255) / 256;
    if (nsplit > max_split) nsplit = max_split;
    const long fit = (long)(part_cap / ((size_t)k1 * k2));
    if (nsplit > fit) nsplit = fit;
    if (nsplit < 1) return GCGE_GPU_ERR_ARG;
    long rps = ((n + nsplit - 1) / nsplit + 31) / 32 * 32;
    if (rps < 32) rps = 32;
    nsplit = (n + rps - 1) / rps;
    if (nsplit < 1) nsplit = 1;
    dim3 grid(ti, tj, (unsigned)nsplit);
    k_gram_partial<<<grid, 256, 0, stream>>>(n, k1, k2, V, ldv, W, ldw, part, rps, sym);
    if (cudaGetLastError() != cudaSuccess) return GCGE_GPU_ERR_CUDA;
    long g = ((long)k1 * k2 + 255) / 256;
    if (g > (long)num_sms * 16) g = (long)num_sms * 16;
    k_gram_reduce<<<(int)(g > 0 ? g : 1), 256, 0, stream>>>(k1, k2, (int)nsplit, part, a_dev, lda, sym);
    if (cudaGetLastError() != cudaSuccess) return GCGE_GPU_ERR_CUDA;
    return GCGE_GPU_OK;
}

// second stage of a Gram product whose per-split partials are already in part
extern "C" int gb_gram_reduce_launch(gcge_gpu_ctx *ctx, int k1, int k2, int nsplit, const double *part,
                                     double *a_dev, int lda, int sym)
{
    GB_LAUNCH(ctx, k_gram_reduce, elem_grid(ctx, (long)k1 * k2), 256, 0, k1, k2, nsplit, part, a_dev, lda, sym);
    return GCGE_GPU_OK;
}
