// gb_ozaki.cu -- FP64-accurate dense contractions of the solver on bf16 tensor cores.
//
// GB300 runs FP64 at ~1.2 TFLOP/s (FP64 tensor MMA no faster) while its bf16
// tensor cores run hundreds of times faster. The two dense contractions of the
// solver -- the Gram product V^T W and the linear combination X C -- therefore
// use an error-free splitting in the style of the Ozaki scheme (Ozaki, Ogita,
// Oishi, Rump, Numer. Algorithms 59, 2012), restated here:
//
//  * every FP64 entry is written against a power-of-two scale of its row or
//    column (gb_tc05.h: oz_bias) as seven balanced base-256 digits in
//    [-128, 127], each exact in bf16, with integer operations only;
//  * a product x y is sum_{p,q} d_p d'_q 2^(-8(p+q)) 2^(e + f - 12); the 28
//    digit pairs with p + q <= 6 are kept (the rest lie below 2^-54 of the scale);
//  * all pairs of one level L = p + q share one FP32 accumulator; with at most
//    7 pairs of products of magnitude <= 2^14, sums over <= 146 terms stay
//    below 2^24, so every level accumulator is an exact integer; it is drained
//    every <= 128 terms into exact int64 sums (levels 0-2 and 3-6) that are
//    rounded once to FP64 (oz_to_double).
//
// The result agrees with an FP64 dot product to within one rounding of the
// exact sum plus the 2^-54-of-scale truncation, independent of summation order.
//
// Kernels:
//  * k_gram_oz -- V^T W on mma.sync m16n8k16 (register accumulators, 32 x 32
//    outputs per CTA over a slice of the rows; column scales from a pre-pass);
//  * k_lincomb_tc -- Y = alpha X C + beta Y on tcgen05: 128 rows x 64 columns of
//    Y per CTA, the seven level accumulators (7 x 64 FP32 columns) in TMEM,
//    digit planes of X (split in the CTA with per-row scales) and of C (split
//    once per call by k_lc_coef_split) double-buffered in shared memory as
//    no-swizzle K-major core matrices, one thread issuing the 28-pair MMAs.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gb_internal.h"
#include "gb_tc05.h"

#define OZ_ROWS 64                 // rows per staged chunk of the Gram (exactness bound: 146)
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
            for (long r = warp; r < n; r += nw) e = max(e, oz_exponent(X[r * ldx + c]));
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

// ---------------------------------------------------------------- Gram (mma.sync)
// stage rows [r0, r0+OZ_ROWS) x columns [c0, c0+32) of X as digit planes
// D[digit][col][row] (bf16, OZ_STRIDE per column); rows beyond n and columns
// beyond k are zero
__device__ __forceinline__ void oz_stage(const double *__restrict__ X, long ldx, long n, int k, long r0, int c0,
                                         const int *__restrict__ exps, uint32_t *__restrict__ D)
{
    const int c = threadIdx.x & 31;
    const int col = c0 + c;
    const int e = col < k ? exps[col] : OZ_NO_EXP;
    for (int rp = threadIdx.x >> 5; rp < OZ_ROWS / 2; rp += blockDim.x >> 5) {
        const long r = r0 + 2 * rp;
        const double x0 = (col < k && r < n) ? X[r * ldx + col] : 0.0;
        const double x1 = (col < k && r + 1 < n) ? X[(r + 1) * ldx + col] : 0.0;
        const unsigned long long u0 = oz_bias(x0, e), u1 = oz_bias(x1, e);
#pragma unroll
        for (int p = 0; p < OZ_DIGITS; ++p) D[(p * OZ_TILE + c) * (OZ_STRIDE / 2) + rp] = oz_pack(u0, u1, p);
    }
}

__device__ __forceinline__ void mma_f16(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// grid (tiles_i, tiles_j, splits); part[split][i + j*k1] = FP64 partial of
// sum_r V[r,i] W[r,j] over the split's rows.
__global__ void __launch_bounds__(128)
k_gram_oz(int n, int k1, int k2, const double *__restrict__ V, long ldv, const double *__restrict__ W, long ldw,
          const int *__restrict__ ev, const int *__restrict__ ew, double *__restrict__ part, long rows_per_split,
          int sym)
{
    extern __shared__ __align__(1024) uint8_t lc_smem[];
    uint32_t *Dv = (uint32_t *)lc_smem;                          // [7][32][OZ_STRIDE/2]
    uint32_t *Dw = Dv + OZ_DIGITS * OZ_TILE * (OZ_STRIDE / 2);
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
                    for (int nt = 0; nt < 2; ++nt) mma_f16(acc[p + q][nt], a[p], b[q][nt]);
        }
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float v[OZ_DIGITS];
#pragma unroll
                for (int L = 0; L < OZ_DIGITS; ++L) v[L] = acc[L][nt][q];
                long long h, l;
                oz_levels_to_int(v, h, l);
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
            if (i < k1 && j < k2) P[i + (long)j * k1] = oz_to_double(hi[nt][q], lo[nt][q], ev[i] + ew[j] - 12);
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

// ---------------------------------------------------------------- linear combination (tcgen05)
#define LC_ROWS 128                                  // rows of Y per CTA (MMA M, TMEM lanes)
#define LC_N 64                                      // columns of Y per CTA (TMEM level stride)
#define LC_KS 32                                     // K (columns of X) per pipeline stage
#define LC_CHUNK 4                                   // stages per exact accumulation (K <= 128)
#define LC_APLANE (LC_ROWS * LC_KS * 2)              // bytes of one digit plane of X per stage
#define LC_BPLANE (LC_N * LC_KS * 2)                 // bytes of one digit plane of C per stage
#define LC_STAGE (OZ_DIGITS * (LC_APLANE + LC_BPLANE))
#define LC_HDR 1024
#define LC_SMEM (2 * LC_STAGE + LC_HDR + 4 * LC_MAX_K)
#define LC_OUT_LD (LC_N + 1)                         // doubles per staged output row
#define LC_WARPS 16                                  // warps of the CTA (all drain TMEM)
#define LC_THREADS (32 * LC_WARPS)
#define LC_SPLIT_WARPS (LC_WARPS - 1)                // warps splitting X; the last one issues the MMAs
#define LC_SPLIT_THREADS (32 * LC_SPLIT_WARPS)
#define LC_CORES (LC_ROWS / 8 * LC_KS / 8)           // core matrices of X per stage
#define LC_CORES_PER_WARP ((LC_CORES + LC_SPLIT_WARPS - 1) / LC_SPLIT_WARPS)
#define LC_COLS_PER_WARP (LC_N * 4 / LC_WARPS)       // output columns drained per warp
#define LC_TMEM_COLS 512
#define LC_WAIT_NS 1000000000ull
#define LC_MAX_K 4096                                // inner dimension handled by the tensor-core path

// Core-matrix layout of one digit plane (no swizzle, K-major): the 8-row x
// 8-element core matrix (g, c) -- rows 8g..8g+7, K 8c..8c+7 of the stage --
// occupies bytes [(4g + c) 128, +128), row by row (16 bytes each). K-adjacent
// core matrices are 128 bytes apart, row-group-adjacent ones 512.
#define LC_LBO 128
#define LC_SBO 512

// Inner-dimension equilibration: X C = (X 2^g) (2^-g C) exactly for any integer
// g_i, so with g_i the exponent of row i of C (max_j |C[i, j]| < 2^g_i) the row
// scale of X 2^g measures |X[r, i]| |C[i, :]|, the size of each term's
// contribution, and the error of a row is relative to its largest term (as for
// an FP64 dot product) even when the columns of X differ widely in magnitude
// and C compensates (the triangular solve of a Cholesky QR).
//
// C (k1 x k2, column-major, only i <= j when upper) -> row scales g (all blocks
// compute them; block (0, 0) stores them), column scales F of 2^-g C (block
// (0, jt) stores its 64) and digit planes Bd[jt][stage][digit] of 2^-g C in
// the core-matrix layout (N = 64 rows j, K = 32 entries i per stage).
// grid (stages, column tiles), 256 threads, k1 <= LC_MAX_K.
__global__ void __launch_bounds__(256)
k_lc_coef_split(int k1, int k2, const double *__restrict__ C, int ldc, int upper, int nst, int *__restrict__ g_out,
                int *__restrict__ f_out, uint32_t *__restrict__ Bd)
{
    __shared__ int gs[LC_MAX_K];
    __shared__ int fs[LC_N];
    const int s = blockIdx.x, jt = blockIdx.y, j0 = jt * LC_N;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = warp; i < k1; i += 8) {
        int e = OZ_NO_EXP;
        for (int j = (upper ? i : 0) + lane; j < k2; j += 32) e = max(e, oz_exponent(C[i + (long)j * ldc]));
        e = __reduce_max_sync(0xffffffffu, e);
        if (lane == 0) {
            gs[i] = e;
            if (s == 0 && jt == 0) g_out[i] = e;
        }
    }
    __syncthreads();
    for (int cc = 0; cc < LC_N / 8; ++cc) {
        const int jj = warp * (LC_N / 8) + cc, j = j0 + jj;
        int e = OZ_NO_EXP;
        if (j < k2) {
            const int iend = upper ? min(k1, j + 1) : k1;
            for (int i = lane; i < iend; i += 32) {
                const int ex = oz_exponent(C[i + (long)j * ldc]);
                if (ex != OZ_NO_EXP) e = max(e, ex - gs[i]);
            }
        }
        e = __reduce_max_sync(0xffffffffu, e);
        if (lane == 0) {
            fs[jj] = e;
            if (s == 0 && j < k2) f_out[j] = e;
        }
    }
    __syncthreads();
    uint32_t *out = Bd + (size_t)(jt * nst + s) * OZ_DIGITS * (LC_BPLANE / 4);
    const int n8 = lane >> 2, kp = lane & 3;
    for (int cc = 0; cc < 4; ++cc) {
        const int core = warp * 4 + cc, g = core >> 2, c = core & 3;
        const int jj = g * 8 + n8, j = j0 + jj, i = s * LC_KS + c * 8 + 2 * kp;
        unsigned long long u0 = OZ_BIAS, u1 = OZ_BIAS;
        if (j < k2) {
            if (i < k1 && (!upper || i <= j)) u0 = oz_bias(C[i + (long)j * ldc], fs[jj] + gs[i]);
            if (i + 1 < k1 && (!upper || i + 1 <= j)) u1 = oz_bias(C[i + 1 + (long)j * ldc], fs[jj] + gs[i + 1]);
        }
        const int w = (core * 128 + n8 * 16 + kp * 4) / 4;
#pragma unroll
        for (int q = 0; q < OZ_DIGITS; ++q) out[q * (LC_BPLANE / 4) + w] = oz_pack(u0, u1, q);
    }
}

// Y[r, j0 + j] = alpha sum_i X[r, i] C[i, j0 + j] + beta Y[r, j0 + j];
// grid (ceil(n / 128), column tiles), LC_THREADS threads, LC_SMEM dynamic shared
// memory. Warp specialised: warps 0 .. LC_SPLIT_WARPS-1 split X into the
// double-buffered stage planes; lane 0 of the last warp issues the MMAs; at the
// end of every chunk all warps drain TMEM (warp w: lanes 32 (w % 4) .. +31, i.e.
// rows, and LC_COLS_PER_WARP columns from LC_COLS_PER_WARP (w / 4)). Hand-offs
// go through mbarriers:
//   full[b]  -- stage planes of buffer b written (LC_SPLIT_THREADS arrivals),
//   empty[b] -- MMAs reading buffer b done (tcgen05.commit),
//   drained  -- TMEM read out after a chunk (LC_THREADS arrivals).
__device__ __forceinline__ void lc_drain(uint32_t trow, int col0, int N, int my_e, const int *ecs, bool first,
                                         double *acc)
{
#pragma unroll
    for (int g8 = 0; g8 < LC_COLS_PER_WARP / 8; ++g8) {
        if (col0 + g8 * 8 < N) {
            uint32_t v[OZ_DIGITS][8];
#pragma unroll
            for (int L = 0; L < OZ_DIGITS; ++L) tc_tmem_ld8(trow + L * LC_N + g8 * 8, v[L]);
            tc_tmem_wait_ld();
#pragma unroll
            for (int L = 0; L < OZ_DIGITS; ++L) tc_reg_fence8(v[L]);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float lev[OZ_DIGITS];
#pragma unroll
                for (int L = 0; L < OZ_DIGITS; ++L) lev[L] = __uint_as_float(v[L][q]);
                long long hi, lo;
                oz_levels_to_int(lev, hi, lo);
                const double d = oz_to_double(hi, lo, my_e + ecs[col0 + g8 * 8 + q] - 12);
                acc[g8 * 8 + q] = first ? d : acc[g8 * 8 + q] + d;
            }
        }
    }
}

__global__ void __launch_bounds__(LC_THREADS, 1)
k_lincomb_tc(int n, int k1, int k2, const double *__restrict__ X, long ldx, const uint4 *__restrict__ Bd,
             const int *__restrict__ g_in, const int *__restrict__ ec, double alpha, double beta,
             double *__restrict__ Y, long ldy, int nst, int *__restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t lc_smem[];
    uint8_t *sm = lc_smem;
    if (*(volatile int *)err) return;                    // an earlier launch timed out: do nothing
    uint64_t *bar = (uint64_t *)(sm + 2 * LC_STAGE);     // full[2], empty[2], drained
    uint32_t *tmem_slot = (uint32_t *)(bar + 5);
    int *sflag = (int *)(tmem_slot + 1);
    int *er = sflag + 1;                                 // [LC_ROWS] row scales of X 2^g
    int *ecs = er + LC_ROWS;                             // [LC_N] column scales of 2^-g C
    int *gs = (int *)(sm + 2 * LC_STAGE + LC_HDR);       // [k1] inner-dimension scales g
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long row0 = (long)blockIdx.x * LC_ROWS;
    const int jt = blockIdx.y, j0 = jt * LC_N;
    const int N = min(LC_N, (k2 - j0 + 15) & ~15);       // MMA width: multiple of 16
    const uint32_t full0 = tc_smem_addr(bar), empty0 = full0 + 16, drained = full0 + 32;

    if (warp == 0) tc_tmem_alloc(tc_smem_addr(tmem_slot), LC_TMEM_COLS);
    if (tid == 0) {
        tc_mbar_init(full0, LC_SPLIT_THREADS);
        tc_mbar_init(full0 + 8, LC_SPLIT_THREADS);
        tc_mbar_init(empty0, 1);
        tc_mbar_init(empty0 + 8, 1);
        tc_mbar_init(drained, LC_THREADS);
        *sflag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < k1; i += LC_THREADS) gs[i] = g_in[i];
    if (tid < LC_N) ecs[tid] = j0 + tid < k2 ? ec[j0 + tid] : OZ_NO_EXP;
    __syncthreads();
    // row scales of X 2^g: warp w, rows w, w + LC_WARPS, ...; four rows in flight
    for (int rr = warp; rr < LC_ROWS; rr += 4 * LC_WARPS) {
        int e[4] = {OZ_NO_EXP, OZ_NO_EXP, OZ_NO_EXP, OZ_NO_EXP};
        for (int i = lane; i < k1; i += 32) {
            const int gi = gs[i];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long r = row0 + rr + q * LC_WARPS;
                if (r < n) {
                    const int ex = oz_exponent(X[r * ldx + i]);
                    if (ex != OZ_NO_EXP && gi != OZ_NO_EXP) e[q] = max(e[q], ex + gi);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int m = __reduce_max_sync(0xffffffffu, e[q]);
            if (lane == 0) er[rr + q * LC_WARPS] = m;
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const uint32_t sbase = tc_smem_addr(sm);
    const int quarter = warp & 3, cgrp = warp >> 2;      // TMEM lane quarter, column group
    const int my_row = quarter * 32 + lane;
    const int col0 = cgrp * LC_COLS_PER_WARP;
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + col0;
    const int my_e = er[my_row];
    double acc[LC_COLS_PER_WARP];
#pragma unroll
    for (int q = 0; q < LC_COLS_PER_WARP; ++q) acc[q] = 0.0;
    int mma_commits[2] = {0, 0};
    const bool mma_warp = warp == LC_SPLIT_WARPS;

    for (int s = 0; s < nst; ++s) {
        const int buf = s & 1, cs = s % LC_CHUNK;
        const bool chunk_end = cs == LC_CHUNK - 1 || s == nst - 1;
        if (mma_warp) {
            // ---------------- MMA issue (one thread)
            if (lane == 0) {
                bool ok = tc_mbar_wait(full0 + 8 * buf, (s >> 1) & 1, LC_WAIT_NS);
                if (ok && cs == 0 && s > 0) ok = tc_mbar_wait(drained, (s / LC_CHUNK - 1) & 1, LC_WAIT_NS);
                if (!ok || *(volatile int *)sflag) {
                    *sflag = 1;
                    atomicExch(err, 1);
                } else {
                    tc_fence_after_sync();
                    const uint32_t a0 = sbase + buf * LC_STAGE, b0 = a0 + OZ_DIGITS * LC_APLANE;
                    const uint32_t idesc = tc_idesc_f16(LC_ROWS, N);
#pragma unroll
                    for (int ks = 0; ks < LC_KS / 16; ++ks)
#pragma unroll
                        for (int p = 0; p < OZ_DIGITS; ++p) {
                            const uint64_t ad = tc_sdesc(a0 + p * LC_APLANE + ks * 256, LC_LBO, LC_SBO);
#pragma unroll
                            for (int q = 0; q + p < OZ_DIGITS; ++q) {
                                const uint64_t bd = tc_sdesc(b0 + q * LC_BPLANE + ks * 256, LC_LBO, LC_SBO);
                                tc_mma_kf16(tmem + (p + q) * LC_N, ad, bd, idesc,
                                            (cs > 0 || ks > 0 || p > 0) ? 1u : 0u);
                            }
                        }
                    tc_mma_commit(empty0 + 8 * buf);
                    ++mma_commits[buf];
                }
            }
            __syncwarp();
        } else {
            // ---------------- split X and copy the C planes into buffer buf
            if (s >= 2 && !tc_mbar_wait(empty0 + 8 * buf, ((s >> 1) - 1) & 1, LC_WAIT_NS)) {
                *sflag = 1;
                atomicExch(err, 1);
            }
            uint8_t *A = sm + buf * LC_STAGE;
            uint8_t *B = A + OZ_DIGITS * LC_APLANE;
            const int i0 = s * LC_KS;
            const int r8 = lane >> 2, kp = lane & 3;
            double xv[LC_CORES_PER_WARP][2];
#pragma unroll
            for (int cc = 0; cc < LC_CORES_PER_WARP; ++cc) {
                const int core = warp + LC_SPLIT_WARPS * cc, g = core >> 2, c = core & 3;
                const long r = row0 + g * 8 + r8;
                const int i = i0 + c * 8 + 2 * kp;
                const bool in = core < LC_CORES && r < n;
                xv[cc][0] = (in && i < k1) ? X[r * ldx + i] : 0.0;
                xv[cc][1] = (in && i + 1 < k1) ? X[r * ldx + i + 1] : 0.0;
            }
            {
                const uint4 *src = Bd + (size_t)(jt * nst + s) * (OZ_DIGITS * LC_BPLANE / 16);
                uint4 *dst = (uint4 *)B;
                for (int v = tid; v < OZ_DIGITS * LC_BPLANE / 16; v += LC_SPLIT_THREADS) dst[v] = src[v];
            }
#pragma unroll
            for (int cc = 0; cc < LC_CORES_PER_WARP; ++cc) {
                const int core = warp + LC_SPLIT_WARPS * cc, g = core >> 2, c = core & 3;
                if (core < LC_CORES) {
                    const int i = i0 + c * 8 + 2 * kp;
                    const int e = er[g * 8 + r8];
                    // a zero row of C (g = OZ_NO_EXP) contributes nothing: its digits stay zero
                    const int g0 = i < k1 ? gs[i] : OZ_NO_EXP, g1 = i + 1 < k1 ? gs[i + 1] : OZ_NO_EXP;
                    const unsigned long long u0 = g0 != OZ_NO_EXP ? oz_bias(xv[cc][0], e - g0) : OZ_BIAS;
                    const unsigned long long u1 = g1 != OZ_NO_EXP ? oz_bias(xv[cc][1], e - g1) : OZ_BIAS;
                    uint32_t *dst = (uint32_t *)(A + core * 128 + r8 * 16 + kp * 4);
#pragma unroll
                    for (int p = 0; p < OZ_DIGITS; ++p) dst[p * (LC_APLANE / 4)] = oz_pack(u0, u1, p);
                }
            }
            tc_fence_async_smem();
            tc_mbar_arrive(full0 + 8 * buf);
        }
        if (chunk_end) {
            // drain the level accumulators of this chunk into FP64 partials
            if (!tc_mbar_wait(empty0 + 8 * buf, (s >> 1) & 1, LC_WAIT_NS)) {
                *sflag = 1;
                atomicExch(err, 1);
            }
            if (*(volatile int *)sflag) break;
            tc_fence_after_sync();
            lc_drain(trow, col0, N, my_e, ecs, s < LC_CHUNK, acc);
            tc_fence_before_sync();
            tc_mbar_arrive(drained);
        }
        if (*(volatile int *)sflag) break;
    }

    __syncthreads();
    if (!*(volatile int *)sflag) {
        // stage the 128 x N block in shared memory (every MMA is done, the operand
        // buffers are idle), then write Y row by row, coalesced
        double *O = (double *)sm;
#pragma unroll
        for (int q = 0; q < LC_COLS_PER_WARP; ++q) O[my_row * LC_OUT_LD + col0 + q] = acc[q];
        __syncthreads();
        const int ncol = min(LC_N, k2 - j0);
        const bool plain = beta == 0.0 && (alpha == 1.0 || alpha == -1.0);
        for (int rr = warp; rr < LC_ROWS; rr += LC_WARPS) {
            const long r = row0 + rr;
            if (r >= n) break;
            for (int q = lane; q < ncol; q += 32) {
                double *y = Y + r * ldy + j0 + q;
                const double v = O[rr * LC_OUT_LD + q];
                *y = plain ? (alpha == 1.0 ? v : -v) : fma(beta, *y, alpha * v);
            }
        }
    }
    // release: after a timeout, wait (bounded) for the MMAs still in flight
    __syncthreads();
    if (mma_warp && lane == 0 && *(volatile int *)sflag) {
        if (mma_commits[0]) tc_mbar_wait(empty0, (mma_commits[0] - 1) & 1, LC_WAIT_NS);
        if (mma_commits[1]) tc_mbar_wait(empty0 + 8, (mma_commits[1] - 1) & 1, LC_WAIT_NS);
    }
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after_sync();
        tc_tmem_dealloc(tmem, LC_TMEM_COLS);
    }
}

extern "C" int gb_lincomb_tc_ok(int k1) { return k1 <= LC_MAX_K; }

extern "C" int gb_lincomb_tc(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *X, long ldx, const double *C,
                             int ldc, double alpha, double beta, double *Y, long ldy, int upper)
{
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_lincomb_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, LC_SMEM) != cudaSuccess)
            return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        attr = true;
    }
    const int nst = (k1 + LC_KS - 1) / LC_KS, jtiles = (k2 + LC_N - 1) / LC_N;
    const size_t bd_bytes = (size_t)jtiles * nst * OZ_DIGITS * LC_BPLANE;
    int st = gb_ozbuf(ctx, bd_bytes);
    if (!st) st = gb_iscratch(ctx, (size_t)k1 + k2);
    if (st) return st;
    uint32_t *Bd = (uint32_t *)ctx->ozbuf;
    int *g = ctx->iscratch, *ec = ctx->iscratch + k1;
    GB_LAUNCH(ctx, k_lc_coef_split, dim3(nst, jtiles), 256, 0, k1, k2, C, ldc, upper, nst, g, ec, Bd);
    GB_PROF(ctx, GB_K_LINCOMB, 8.0 * n * k1 + (beta != 0.0 ? 16.0 : 8.0) * n * k2,
            upper ? 1.0 * n * k1 * (k2 + 1) : 2.0 * n * k1 * k2);
    GB_LAUNCH(ctx, k_lincomb_tc, dim3((unsigned)((n + LC_ROWS - 1) / LC_ROWS), jtiles), LC_THREADS, LC_SMEM, n, k1, k2, X,
              ldx, (const uint4 *)Bd, g, ec, alpha, beta, Y, ldy, nst, ctx->dev_err);
    return GCGE_GPU_OK;
}
