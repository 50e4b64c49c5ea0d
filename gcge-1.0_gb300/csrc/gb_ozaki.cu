// gb_ozaki.cu -- FP64-accurate tall-skinny products on bf16 tensor cores.
//
// GB300 runs FP64 at 1.2 TFLOP/s (FP64 tensor MMA no faster) but bf16 mma.sync at
// ~600 TFLOP/s. The Gram product V^T W of the solver is therefore computed with
// an error-free splitting in the style of the Ozaki scheme (Ozaki, Ogita, Oishi,
// Rump, Numer. Algorithms 59, 2012), restated here for this kernel:
//
//  * every FP64 entry x of column i is written against a power-of-two scale
//    2^e_i (|x| < 2^e_i for the whole column) as the integer T = x 2^(55 - e_i)
//    (|T| < 2^55, exact down to 2^(e_i - 55)), and T is split into seven balanced
//    base-256 digits d_0..d_6 in [-128, 128] (T = sum_p d_p 2^(48 - 8p)) -- with
//    integer bit operations only, no FP64 arithmetic; each digit is exact in bf16;
//  * a product x y is sum_{p,q} d_p d'_q 2^(-8(p+q)) 2^(e_i + f_j - 14); the 28
//    digit pairs with p + q <= 6 are kept (the rest lie below 2^-56 of the scale);
//  * pairs of one level L = p + q share one FP32 accumulator; with at most 7
//    pairs of products of magnitude <= 2^14, 64 rows sum to < 2^24, so every
//    level accumulator is an exact integer; it is flushed every 64 rows into two
//    exact int64 accumulators (levels 0-2 and 3-6);
//  * the int64 totals are turned into FP64 once per output.
//
// The result agrees with an FP64 dot product to within FP64 rounding of the
// partial sums (plus the 2^-56-of-scale truncation), independent of row order.
//
// Tiling: 128-thread CTAs, 2 x 2 warps, each warp a 16 (i) x 16 (j) block of
// outputs as two m16n8k16 tiles; a CTA covers 32 x 32 outputs over a slice of
// the rows, staged 64 rows at a time as bf16 digit planes in shared memory
// (layout [digit][column][row], rows contiguous, so every mma fragment is one
// 32-bit shared load). Per-split FP64 partials are summed by k_gram_reduce
// (gb_blas.cu) in a fixed order.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gb_internal.h"

#define OZ_DIGITS 7
#define OZ_ROWS 64                 // rows per staged chunk (exactness bound: 146)
#define OZ_STRIDE (OZ_ROWS + 4)    // bf16 per staged column (34 words: 2-way banks)
#define OZ_TILE 32
#define OZ_MAX_SPLIT_ROWS (1L << 20)

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

extern "C" int gb_gram_reduce_launch(gcge_gpu_ctx *ctx, int k1, int k2, int nsplit, const double *part,
                                     double *a_dev, int lda, int sym);

// ---------------------------------------------------------------- scales
#define OZ_NO_EXP (-2000)          // exponent of an all-zero column

// exps[c] = smallest e with |X[r, c]| < 2^e for all rows (OZ_NO_EXP for an
// all-zero column; subnormal entries count as zero). exps must hold OZ_NO_EXP
// on entry; each block reduces its rows first and issues one atomic per column.
__global__ void __launch_bounds__(256)
k_col_exponent(int n, int k, const double *__restrict__ X, long ldx, int *__restrict__ exps)
{
    __shared__ int se[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (int c0 = 0; c0 < k; c0 += 32) {
        const int c = c0 + lane;
        int e = OZ_NO_EXP;
        if (c < k)
            for (long r = warp; r < n; r += nw) {
                const long long b = __double_as_longlong(X[r * ldx + c]);
                const int ex = (int)((b >> 52) & 0x7ff);
                if (ex) e = max(e, ex - 1022);    // |x| < 2^(ex - 1022)
            }
        se[w][lane] = e;
        __syncthreads();
        if (w == 0) {
#pragma unroll
            for (int q = 1; q < 8; ++q) e = max(e, se[q][lane]);
            if (c < k && e > OZ_NO_EXP) atomicMax(exps + c, e);
        }
        __syncthreads();
    }
}

__global__ void k_fill_int(int *p, int count, int v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) p[i] = v;
}

// ---------------------------------------------------------------- splitting
// seven balanced base-256 digits of T = x 2^(55 - e) (|x| < 2^e)
__device__ __forceinline__ void oz_digits(double x, int e, int d[OZ_DIGITS])
{
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    long long T = 0;
    if (ex) {
        const long long mant = (b & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
        const int sh = ex - 1020 - e;                 // T = mant 2^sh, sh <= 2
        if (sh >= 0) T = mant << sh;
        else if (sh > -62) T = (mant + (1LL << (-sh - 1))) >> (-sh);
        if (b < 0) T = -T;
    }
#pragma unroll
    for (int p = 0; p < OZ_DIGITS - 1; ++p) {
        const int s = 48 - 8 * p;
        const long long q = (T + (1LL << (s - 1))) >> s;   // round to nearest (ties up)
        d[p] = (int)q;
        T -= q << s;
    }
    d[OZ_DIGITS - 1] = (int)T;
}

__device__ __forceinline__ uint32_t pack_bf16x2(int lo, int hi)
{
    const __nv_bfloat16 a = __float2bfloat16_rn((float)lo), b = __float2bfloat16_rn((float)hi);
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// stage rows [r0, r0+OZ_ROWS) x columns [c0, c0+32) of X as digit planes
// D[digit][col][row] (bf16, OZ_STRIDE per column); rows beyond n and columns
// beyond k are zero
__device__ __forceinline__ void oz_stage(const double *__restrict__ X, long ldx, long n, int k, long r0, int c0,
                                         const int *__restrict__ exps, uint32_t *__restrict__ D)
{
    const int c = threadIdx.x & 31;
    const int col = c0 + c;
    const int e = col < k ? exps[col] : 0;
    for (int rp = threadIdx.x >> 5; rp < OZ_ROWS / 2; rp += blockDim.x >> 5) {
        const long r = r0 + 2 * rp;
        int d0[OZ_DIGITS], d1[OZ_DIGITS];
        const double x0 = (col < k && r < n) ? X[r * ldx + col] : 0.0;
        const double x1 = (col < k && r + 1 < n) ? X[(r + 1) * ldx + col] : 0.0;
        oz_digits(x0, e, d0);
        oz_digits(x1, e, d1);
#pragma unroll
        for (int p = 0; p < OZ_DIGITS; ++p)
            D[(p * OZ_TILE + c) * (OZ_STRIDE / 2) + rp] = pack_bf16x2(d0[p], d1[p]);
    }
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ---------------------------------------------------------------- Gram
// grid (tiles_i, tiles_j, splits); part[split][i + j*k1] = FP64 partial of
// sum_r V[r,i] W[r,j] over the split's rows.
__global__ void __launch_bounds__(128)
k_gram_oz(int n, int k1, int k2, const double *__restrict__ V, long ldv, const double *__restrict__ W, long ldw,
          const int *__restrict__ ev, const int *__restrict__ ew, double *__restrict__ part, long rows_per_split,
          int sym)
{
    extern __shared__ uint32_t sm[];
    uint32_t *Dv = sm;                                           // [7][32][OZ_STRIDE/2]
    uint32_t *Dw = sm + OZ_DIGITS * OZ_TILE * (OZ_STRIDE / 2);
    const int ti = blockIdx.x, tj = blockIdx.y;
    if (sym && ti > tj) return;
    const int i0 = ti * OZ_TILE, j0 = tj * OZ_TILE;
    const long rb = (long)blockIdx.z * rows_per_split;
    const long re = min((long)n, rb + rows_per_split);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wi = (warp >> 1) * 16, wj = (warp & 1) * 16;     // warp tile origin inside the CTA tile
    const int g = lane >> 2, t = lane & 3;
    float acc[OZ_DIGITS][2][4];
    long long hi[2][4], lo[2][4];
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) { hi[nt][q] = 0; lo[nt][q] = 0; }
    for (long r0 = rb; r0 < re; r0 += OZ_ROWS) {
        __syncthreads();
        oz_stage(V, ldv, re, k1, r0, i0, ev, Dv);
        oz_stage(W, ldw, re, k2, r0, j0, ew, Dw);
        __syncthreads();
#pragma unroll
        for (int L = 0; L < OZ_DIGITS; ++L)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[L][nt][q] = 0.f;
#pragma unroll 1
        for (int k0 = 0; k0 < OZ_ROWS; k0 += 16) {
            const int kw = k0 / 2 + t;                           // 32-bit word of rows k0+2t, k0+2t+1
            uint32_t a[OZ_DIGITS][4], b[OZ_DIGITS][2][2];
#pragma unroll
            for (int p = 0; p < OZ_DIGITS; ++p) {
                const uint32_t *A0 = Dv + (p * OZ_TILE + wi + g) * (OZ_STRIDE / 2);
                const uint32_t *A8 = Dv + (p * OZ_TILE + wi + g + 8) * (OZ_STRIDE / 2);
                a[p][0] = A0[kw];
                a[p][1] = A8[kw];
                a[p][2] = A0[kw + 4];
                a[p][3] = A8[kw + 4];
#pragma unroll
                for (int nt = 0; nt < 2; ++nt) {
                    const uint32_t *B0 = Dw + (p * OZ_TILE + wj + nt * 8 + g) * (OZ_STRIDE / 2);
                    b[p][nt][0] = B0[kw];
                    b[p][nt][1] = B0[kw + 4];
                }
            }
#pragma unroll
            for (int p = 0; p < OZ_DIGITS; ++p)
#pragma unroll
                for (int q = 0; q + p < OZ_DIGITS; ++q)
#pragma unroll
                    for (int nt = 0; nt < 2; ++nt) mma_bf16(acc[p + q][nt], a[p], b[q][nt]);
        }
        // flush: level L carries weight 2^(-8L); hi collects levels 0-2 in units of
        // 2^-16, lo levels 3-6 in units of 2^-48 (all exact integers)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                long long h = 0, l = 0;
#pragma unroll
                for (int L = 0; L < 3; ++L) h += (long long)__float2int_rn(acc[L][nt][q]) << (8 * (2 - L));
#pragma unroll
                for (int L = 3; L < OZ_DIGITS; ++L) l += (long long)__float2int_rn(acc[L][nt][q]) << (8 * (6 - L));
                hi[nt][q] += h;
                lo[nt][q] += l;
            }
    }
    // C fragment: c0,c1 -> row g, cols 2t, 2t+1; c2,c3 -> row g+8
    double *P = part + (long)blockIdx.z * k1 * k2;
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = i0 + wi + g + (q >= 2 ? 8 : 0);
            const int j = j0 + wj + nt * 8 + 2 * t + (q & 1);
            if (i < k1 && j < k2) {
                const int s = ev[i] + ew[j] - 14;
                P[i + (long)j * k1] = ldexp((double)hi[nt][q], s - 16) + ldexp((double)lo[nt][q], s - 48);
            }
        }
}

static size_t oz_smem() { return 2u * OZ_DIGITS * OZ_TILE * (OZ_STRIDE / 2) * sizeof(uint32_t); }

// a[i + j*lda] = sum_r V[r,i] W[r,j] to FP64 accuracy on the tensor cores.
// exps: device int[k1 + k2] scratch for the column scales.
extern "C" int gb_gram_tc(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *V, long ldv, const double *W,
                          long ldw, double *a_dev, int lda, int sym, int *exps)
{
    if (k1 <= 0 || k2 <= 0) return GCGE_GPU_OK;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_gram_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_smem()) !=
            cudaSuccess)
            return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        attr = true;
    }
    const int ti = (k1 + OZ_TILE - 1) / OZ_TILE, tj = (k2 + OZ_TILE - 1) / OZ_TILE;
    int tiles = sym ? ti * (ti + 1) / 2 : ti * tj;
    if (tiles < 1) tiles = 1;
    long nsplit = ((long)ctx->num_sms * 8) / tiles;
    const long max_split = (n + 2047) / 2048;
    if (nsplit > max_split) nsplit = max_split;
    // int64 headroom: a row adds < 2^41 to lo (levels 3-6 in units of 2^-48),
    // so a split holds at most 2^20 rows
    const long min_split = (n + OZ_MAX_SPLIT_ROWS - 1) / OZ_MAX_SPLIT_ROWS;
    if (nsplit < min_split) nsplit = min_split;
    if (nsplit < 1) nsplit = 1;
    long rps = ((n + nsplit - 1) / nsplit + OZ_ROWS - 1) / OZ_ROWS * OZ_ROWS;
    nsplit = (n + rps - 1) / rps;
    if (nsplit < 1) nsplit = 1;
    int st = gb_scratch(ctx, (size_t)nsplit * k1 * k2);
    if (st) return st;
    GB_LAUNCH(ctx, k_fill_int, (k1 + k2 + 127) / 128, 128, 0, exps, k1 + k2, OZ_NO_EXP);
    const int eg = ctx->num_sms * 4;
    GB_LAUNCH(ctx, k_col_exponent, eg, 256, 0, n, k1, V, ldv, exps);
    GB_LAUNCH(ctx, k_col_exponent, eg, 256, 0, n, k2, W, ldw, exps + k1);
    dim3 grid(ti, tj, (unsigned)nsplit);
    GB_PROF(ctx, GB_K_GRAM, 8.0 * n * (k1 + k2), sym ? 1.0 * n * k1 * (k1 + 1) : 2.0 * n * k1 * k2);
    GB_LAUNCH(ctx, k_gram_oz, grid, 128, oz_smem(), n, k1, k2, V, ldv, W, ldw, exps, exps + k1, ctx->scratch, rps,
              sym);
    return gb_gram_reduce_launch(ctx, k1, k2, (int)nsplit, ctx->scratch, a_dev, lda, sym);
}
