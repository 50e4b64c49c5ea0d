// gb_ozaki.cu -- FP64-accurate dense contractions of the solver on the tcgen05
// tensor cores.
//
// GB300 runs FP64 at ~1.2 TFLOP/s (FP64 tensor MMA no faster) while its f16
// tensor cores run at ~2 PFLOP/s. The two dense contractions of the solver -- the
// Gram product V^T W and the linear combination X C -- therefore use an
// error-free splitting in the style of the Ozaki scheme (Ozaki, Ogita, Oishi,
// Rump, Numer. Algorithms 59, 2012), restated here:
//
//  * every FP64 entry is written against a power-of-two scale of its row or
//    column (gb_tc05.h: oz_bias) as seven balanced base-256 digits, each exact
//    in f16, with integer operations only;
//  * a product x y is sum_{p,q} d_p d'_q 2^(-8(p+q)) 2^(e + f - 10); the digit
//    pairs of levels p + q < 8 are kept (34 pairs; the dropped ones lie below
//    2^-57 of the scale product per term);
//  * all pairs of one level L = p + q share one FP32 accumulator in TMEM, which
//    stays an exact integer for up to OZ_EXACT_TERMS terms; it is drained at
//    most every OZ_EXACT_TERMS terms into exact int64 sums (levels 0-2 and the
//    lower ones) that are rounded once to FP64 (oz_to_double).
//
// Both kernels share one structure (tcgen05, 128 x 64 output tile per CTA):
//  * 16 warps, one CTA per SM; warps 0-14 split FP64 operands into f16 digit
//    planes in shared memory (two stages of K = 32, no-swizzle K-major core
//    matrices), lane 0 of warp 15 issues the digit-pair MMAs of a stage
//    (M = 128, N = 64, K = 16, accumulators: 8 levels x 64 TMEM columns), and
//    all 16 warps drain TMEM (warp w: lanes 32 (w % 4) .. +31, 16 columns from
//    16 (w / 4));
//  * hand-offs through mbarriers: full[b] (stage b written, 480 arrivals),
//    empty[b] (MMAs of stage b done, tcgen05.commit), drained (TMEM read out,
//    512 arrivals), copied[b] (bulk copy of the pre-split planes of stage b);
//    every wait is bounded and reports a timeout through the context's device
//    error word;
//  * the split warps load the next stage's FP64 values while the MMAs of the
//    current one run.
// k_lincomb_tc: Y = alpha X C + beta Y, M = 128 rows of X, K = columns of X,
//   per-row scales (of X equilibrated by the row scales of C), C split once per
//   call by k_lc_coef_split;
// k_gram_tc: V^T W, M = 128 columns of V, N = 64 columns of W, K = rows of a
//   row split, per-column scales from a pre-pass (k_col_exponent); partial
//   Grams of the splits are summed in a fixed order by k_gram_reduce.
#include <cstdint>
#include <cuda_runtime.h>

#include "gb_internal.h"
#include "gb_tc05.h"

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

// ---------------------------------------------------------------- tile geometry
#define TC_M 128                                     // MMA M, TMEM lanes
#define TC_N 64                                      // MMA N (max), TMEM columns per level
#define TC_KS 32                                     // K per pipeline stage
#define TC_APLANE (TC_M * TC_KS * 2)                 // bytes of one f16 digit plane, A operand
#define TC_BPLANE (TC_N * TC_KS * 2)                 // bytes of one f16 digit plane, B operand
#define TC_STAGE (OZ_DIGITS * (TC_APLANE + TC_BPLANE))
#define TC_HDR 1024                                  // mbarriers, TMEM address, flags, scales
#define TC_WARPS 16
#define TC_THREADS (32 * TC_WARPS)
#define TC_SPLIT_WARPS (TC_WARPS - 1)
#define TC_SPLIT_THREADS (32 * TC_SPLIT_WARPS)
#define TC_ACORES (TC_M / 8 * TC_KS / 8)             // core matrices of the A operand per stage
#define TC_BCORES (TC_N / 8 * TC_KS / 8)
#define TC_COLS_PER_WARP (TC_N * 4 / TC_WARPS)       // output columns drained per warp (16)
#define TC_TMEM_COLS 512
#define TC_WAIT_NS 1000000000ull
// Core-matrix layout of one digit plane (no swizzle, K-major): the 8-row x
// 8-element core matrix (g, c) -- rows 8g..8g+7, K 8c..8c+7 of the stage --
// occupies bytes [(4g + c) 128, +128), row by row (16 bytes each). K-adjacent
// core matrices are 128 bytes apart, row-group-adjacent ones 512.
#define TC_LBO 128
#define TC_SBO 512
// stages per exact accumulation when the K range is longer than OZ_EXACT_TERMS
#define TC_CHUNK_STAGES (OZ_EXACT_TERMS / TC_KS)

// shared header of both kernels
struct tc_hdr {
    uint64_t bar[7];             // full[2], empty[2], drained, copied[2] (bulk copies of a stage)
    uint32_t tmem;
    int flag;                    // a bounded wait ran out in this CTA
};
static_assert(sizeof(tc_hdr) <= 64, "header overlaps the scale arrays");

__device__ __forceinline__ void tc_fail(tc_hdr *h, int *err)
{
    h->flag = 1;
    atomicExch(err, 1);
}

// CTA start: TMEM allocation (warp 0), mbarrier initialisation (thread 0)
__device__ __forceinline__ void tc_setup(tc_hdr *h)
{
    if ((threadIdx.x >> 5) == 0) tc_tmem_alloc(tc_smem_addr(&h->tmem), TC_TMEM_COLS);
    if (threadIdx.x == 0) {
        const uint32_t b = tc_smem_addr(h->bar);
        tc_mbar_init(b, TC_SPLIT_THREADS);
        tc_mbar_init(b + 8, TC_SPLIT_THREADS);
        tc_mbar_init(b + 16, 1);
        tc_mbar_init(b + 24, 1);
        tc_mbar_init(b + 32, TC_THREADS);
        tc_mbar_init(b + 40, 1);
        tc_mbar_init(b + 48, 1);
        h->flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

// MMA issue of stage s (lane 0 of the MMA warp): wait for the stage's planes
// (and, at the first stage of a chunk, for the previous chunk's drain), issue the
// digit pairs with p + q < LEVELS x TC_KS / 16 K steps, commit to empty[buf].
// The B digit planes of a stage lie back to back with the same 512-byte stride
// between 8-row groups, and level L of the accumulator is TMEM columns 64 L ..
// 64 L + 63, so the pairs (p, q0) .. (p, q0 + 3) are one MMA with N = 64 x 4
// whose D starts at level p + q0: 11 MMAs per K step (10 for the Gram's seven
// levels) instead of 34 (28), and each A plane is read from shared memory once
// per such group instead of once per pair. The first K step of a chunk keeps
// the pairwise order, whose first MMA into every level overwrites it.
// stall (test hook, GCGE_GPU_TestStallTensorWait): before the first stage the
// issuing thread waits for the first drain, an arrival that cannot come before
// the MMAs it would issue, so that bounded wait runs out and the CTA takes the
// timeout path (no MMA is issued; the other warps' waits run out in turn).
template <int LEVELS, bool COPIED>
__device__ __forceinline__ void tc_issue_stage(tc_hdr *h, uint32_t sbase, uint32_t tmem, int N, int s, int cs,
                                               int *commits, int *err, int stall)
{
    const int buf = s & 1;
    const uint32_t full = tc_smem_addr(h->bar) + 8 * buf, empty = tc_smem_addr(h->bar) + 16 + 8 * buf;
    const uint32_t drained = tc_smem_addr(h->bar) + 32, copied = tc_smem_addr(h->bar) + 40 + 8 * buf;
    if (stall && s == 0 && !tc_mbar_wait(drained, 0, TC_WAIT_NS)) {
        tc_fail(h, err);
        return;
    }
    bool ok = tc_mbar_wait(full, (s >> 1) & 1, TC_WAIT_NS);
    if (COPIED && ok) ok = tc_mbar_wait(copied, (s >> 1) & 1, TC_WAIT_NS);
    if (ok && cs == 0 && s > 0) ok = tc_mbar_wait(drained, (commits[2] - 1) & 1, TC_WAIT_NS);
    if (!ok || *(volatile int *)&h->flag) {
        tc_fail(h, err);
        return;
    }
    tc_fence_after_sync();
    (void)N;
    const uint32_t a0 = sbase + buf * TC_STAGE, b0 = a0 + OZ_DIGITS * TC_APLANE;
    const uint32_t idesc = tc_idesc_f16(TC_M, TC_N);
#pragma unroll
    for (int ks = 0; ks < TC_KS / 16; ++ks) {
        if (cs == 0 && ks == 0) {
#pragma unroll
            for (int p = 0; p < OZ_DIGITS; ++p) {
                const uint64_t ad = tc_sdesc(a0 + p * TC_APLANE, TC_LBO, TC_SBO);
#pragma unroll
                for (int q = 0; q < OZ_DIGITS; ++q) {
                    if (p + q < LEVELS) {
                        const uint64_t bd = tc_sdesc(b0 + q * TC_BPLANE, TC_LBO, TC_SBO);
                        // the first MMA into level L is (p, q) = (max(0, L - 6), min(L, 6))
                        const bool first = p == (p + q > OZ_DIGITS - 1 ? p + q - (OZ_DIGITS - 1) : 0);
                        tc_mma_kf16(tmem + (p + q) * TC_N, ad, bd, idesc, first ? 0u : 1u);
                    }
                }
            }
        } else {
#pragma unroll
            for (int p = 0; p < OZ_DIGITS; ++p) {
                const int qmax = (LEVELS - 1 - p < OZ_DIGITS - 1) ? LEVELS - 1 - p : OZ_DIGITS - 1;
                const uint64_t ad = tc_sdesc(a0 + p * TC_APLANE + ks * 256, TC_LBO, TC_SBO);
#pragma unroll
                for (int q0 = 0; q0 <= qmax; q0 += 4) {
                    const int nq = qmax - q0 + 1 < 4 ? qmax - q0 + 1 : 4;
                    const uint64_t bd = tc_sdesc(b0 + q0 * TC_BPLANE + ks * 256, TC_LBO, TC_SBO);
                    tc_mma_kf16(tmem + (p + q0) * TC_N, ad, bd, tc_idesc_f16(TC_M, TC_N * nq), 1u);
                }
            }
        }
    }
    tc_mma_commit(empty);
    ++commits[buf];
}

// TMEM read-out of 4 columns x LEVELS levels for this thread's lane (row of the tile)
template <int LEVELS>
__device__ __forceinline__ void tc_load_levels4(uint32_t taddr, uint32_t v[][4])
{
#pragma unroll
    for (int L = 0; L < LEVELS; ++L)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                     : "=r"(v[L][0]), "=r"(v[L][1]), "=r"(v[L][2]), "=r"(v[L][3])
                     : "r"(taddr + L * TC_N));
    tc_tmem_wait_ld();
#pragma unroll
    for (int L = 0; L < LEVELS; ++L) asm volatile("" : "+r"(v[L][0]), "+r"(v[L][1]), "+r"(v[L][2]), "+r"(v[L][3]));
}

// wait for the chunk's last MMAs before the drain
__device__ __forceinline__ bool tc_wait_chunk(tc_hdr *h, int s, int *err)
{
    const uint32_t empty = tc_smem_addr(h->bar) + 16 + 8 * (s & 1);
    if (!tc_mbar_wait(empty, (s >> 1) & 1, TC_WAIT_NS)) tc_fail(h, err);
    if (*(volatile int *)&h->flag) return false;
    tc_fence_after_sync();
    return true;
}

// copies: bulk copies issued per buffer by thread 0 (nullptr if none)
__device__ __forceinline__ void tc_release(tc_hdr *h, uint32_t tmem, int mma_warp, const int *commits,
                                           const int *copies)
{
    __syncthreads();
    if (*(volatile int *)&h->flag) {
        // after a timeout: wait (bounded) for the MMAs and copies still in flight
        if (mma_warp && (threadIdx.x & 31) == 0) {
            const uint32_t e = tc_smem_addr(h->bar) + 16;
            if (commits[0]) tc_mbar_wait(e, (commits[0] - 1) & 1, TC_WAIT_NS);
            if (commits[1]) tc_mbar_wait(e + 8, (commits[1] - 1) & 1, TC_WAIT_NS);
        }
        if (copies && threadIdx.x == 0) {
            const uint32_t c = tc_smem_addr(h->bar) + 40;
            if (copies[0]) tc_mbar_wait(c, (copies[0] - 1) & 1, TC_WAIT_NS);
            if (copies[1]) tc_mbar_wait(c + 8, (copies[1] - 1) & 1, TC_WAIT_NS);
        }
    }
    tc_fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        tc_fence_after_sync();
        tc_tmem_dealloc(tmem, TC_TMEM_COLS);
    }
}

// ---------------------------------------------------------------- Gram column scales
// exps[c] = smallest e with |X[r, c]| < 2^e for all rows (OZ_NO_EXP for an
// all-zero column; subnormal entries count as zero). exps must hold OZ_NO_EXP
// on entry. A warp reads whole rows (lane l: columns c0 + l + 32 j, 8 independent
// loads per row in flight) over 256-column chunks, so each row's bytes stream
// once per chunk; each block reduces its warps and issues one atomic per column.
#define CE_COLS 256
__global__ void __launch_bounds__(256)
k_col_exponent(int n, int k, const double *__restrict__ X, long ldx, int *__restrict__ exps)
{
    __shared__ int se[8][CE_COLS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long warp = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (int c0 = 0; c0 < k; c0 += CE_COLS) {
        int e[CE_COLS / 32];
#pragma unroll
        for (int j = 0; j < CE_COLS / 32; ++j) e[j] = OZ_NO_EXP;
        for (long r = warp; r < n; r += nw) {
            const double *xr = X + r * ldx + c0 + lane;
            double v[CE_COLS / 32];
#pragma unroll
            for (int j = 0; j < CE_COLS / 32; ++j) v[j] = c0 + lane + 32 * j < k ? __ldg(xr + 32 * j) : 0.0;
#pragma unroll
            for (int j = 0; j < CE_COLS / 32; ++j) e[j] = max(e[j], oz_exponent(v[j]));
        }
#pragma unroll
        for (int j = 0; j < CE_COLS / 32; ++j) se[w][lane + 32 * j] = e[j];
        __syncthreads();
        for (int c = threadIdx.x; c < CE_COLS; c += blockDim.x) {
            int m = se[0][c];
#pragma unroll
            for (int q = 1; q < 8; ++q) m = max(m, se[q][c]);
            if (c0 + c < k && m > OZ_NO_EXP) atomicMax(exps + c0 + c, m);
        }
        __syncthreads();
    }
}

__global__ void k_fill_int(int *p, int count, int v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) p[i] = v;
}

// ---------------------------------------------------------------- Gram V^T W (tcgen05)
#define GR_CORES_PER_WARP ((TC_ACORES + TC_BCORES + TC_SPLIT_WARPS - 1) / TC_SPLIT_WARPS)
// Levels 0-7 (34 digit pairs, 8 x 64 TMEM columns), as the linear combination:
// the dropped pairs (level >= 8) add at most 2^-57.4 of the column-scale product
// 2^(e+f) per row, so over n rows the error stays below 2^-57.4 n 2^(e+f) even
// when every row drops the same amount (e.g. constant columns) -- far below the
// FP64 summation error of the same Gram. Levels 3-7 are summed in units of level 7
// (2^-56) and carried into the level 0-2 sum (units 2^-16) after every chunk, so
// neither int64 sum can overflow for the 2^20 rows a split may hold.
#define GR_LEVELS 8
#define GR_SMEM (2 * TC_STAGE + TC_HDR)

// grid (ceil(k1 / 128), ceil(k2 / 64), splits); part[split][i + j k1] = the
// split's exact integer sum of the digit products of sum_r V[r, i] W[r, j] as
// (hi, lo), value (hi 2^40 + lo) 2^(e_i + f_j - 66) (sym: tiles wholly below
// the diagonal are skipped).
__global__ void __launch_bounds__(TC_THREADS, 1)
k_gram_tc(int n, int k1, int k2, const double *__restrict__ V, long ldv, const double *__restrict__ W, long ldw,
          const int *__restrict__ ev, const int *__restrict__ ew, long long *__restrict__ part, long rows_per_split,
          int sym, int *__restrict__ err, int stall)
{
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint8_t *sm = tc_smem;
    const int i0 = blockIdx.x * TC_M, j0 = blockIdx.y * TC_N;
    if (sym && i0 > j0 + TC_N - 1) return;
    if (*(volatile int *)err) return;                    // an earlier launch timed out: do nothing
    tc_hdr *h = (tc_hdr *)(sm + 2 * TC_STAGE);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long rb = (long)blockIdx.z * rows_per_split;
    const long re = min((long)n, rb + rows_per_split);
    const int nst = (int)((re - rb + TC_KS - 1) / TC_KS);
    const int N = min(TC_N, (k2 - j0 + 15) & ~15);
    tc_setup(h);
    // digit planes of both buffers start at zero: core matrices wholly outside the
    // columns of V or W (the padding of a short tile) are never split and keep
    // zero digits; the split threads' first proxy fence covers these writes
    if (tid < TC_SPLIT_THREADS)
        for (int i = tid; i < 2 * TC_STAGE / 16; i += TC_SPLIT_THREADS)
            reinterpret_cast<uint4 *>(sm)[i] = make_uint4(0u, 0u, 0u, 0u);
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = h->tmem, sbase = tc_smem_addr(sm);
    const bool mma_warp = warp == TC_SPLIT_WARPS;
    const int quarter = warp & 3, col0 = (warp >> 2) * TC_COLS_PER_WARP;
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + col0;
    int commits[3] = {0, 0, 0};                          // empty[0], empty[1], drained chunks
    long long hi[TC_COLS_PER_WARP], lo[TC_COLS_PER_WARP];
#pragma unroll
    for (int q = 0; q < TC_COLS_PER_WARP; ++q) hi[q] = lo[q] = 0;

    // split-warp geometry: core q = warp + 15 cc; A cores (V) first, then B cores (W);
    // lane (i8, rp): column 8g + i8, rows 8c + 2 rp and 8c + 2 rp + 1
    const int i8 = lane & 7, rp = lane >> 3;
    double xv[GR_CORES_PER_WARP][2];
    auto load_stage = [&](int s) {
        const long r = rb + (long)s * TC_KS + 2 * rp;
#pragma unroll
        for (int cc = 0; cc < GR_CORES_PER_WARP; ++cc) {
            const int q = warp + TC_SPLIT_WARPS * cc;
            const bool isA = q < TC_ACORES;
            const int qq = isA ? q : q - TC_ACORES;
            const int col = (isA ? i0 : j0) + 8 * (qq >> 2) + i8;
            const long rr = r + 8 * (qq & 3);
            const double *src = isA ? V : W;
            const long ld = isA ? ldv : ldw;
            const bool in = q < TC_ACORES + TC_BCORES && col < (isA ? k1 : k2);
            xv[cc][0] = (in && rr < re) ? src[rr * ld + col] : 0.0;
            xv[cc][1] = (in && rr + 1 < re) ? src[(rr + 1) * ld + col] : 0.0;
        }
    };
    if (!mma_warp) load_stage(0);

    for (int s = 0; s < nst; ++s) {
        const int buf = s & 1, cs = s % TC_CHUNK_STAGES;
        const bool chunk_end = cs == TC_CHUNK_STAGES - 1 || s == nst - 1;
        if (mma_warp) {
            if (lane == 0) tc_issue_stage<GR_LEVELS, false>(h, sbase, tmem, N, s, cs, commits, err, stall);
            __syncwarp();
        } else {
            if (s >= 2 && !tc_mbar_wait(tc_smem_addr(h->bar) + 16 + 8 * buf, ((s >> 1) - 1) & 1, TC_WAIT_NS))
                tc_fail(h, err);
            uint8_t *A = sm + buf * TC_STAGE;
            uint8_t *B = A + OZ_DIGITS * TC_APLANE;
#pragma unroll
            for (int cc = 0; cc < GR_CORES_PER_WARP; ++cc) {
                const int q = warp + TC_SPLIT_WARPS * cc;
                const bool isA = q < TC_ACORES;
                const int qq = isA ? q : q - TC_ACORES;
                if (q < TC_ACORES + TC_BCORES && (isA ? i0 : j0) + 8 * (qq >> 2) < (isA ? k1 : k2)) {
                    const int col = (isA ? i0 : j0) + 8 * (qq >> 2) + i8;
                    const int e = col < (isA ? k1 : k2) ? (isA ? ev : ew)[col] : OZ_NO_EXP;
                    const unsigned long long u0 = oz_bias(xv[cc][0], e), u1 = oz_bias(xv[cc][1], e);
                    uint32_t *dst = (uint32_t *)((isA ? A : B) + qq * 128 + i8 * 16 + rp * 4);
                    const int pl = (isA ? TC_APLANE : TC_BPLANE) / 4;
#pragma unroll
                    for (int p = 0; p < OZ_DIGITS; ++p) dst[p * pl] = oz_pack(u0, u1, p);
                }
            }
            tc_fence_async_smem();
            tc_mbar_arrive(tc_smem_addr(h->bar) + 8 * buf);
            if (s + 1 < nst) load_stage(s + 1);          // in flight while the MMAs run
        }
        if (chunk_end) {
            if (!tc_wait_chunk(h, s, err)) break;
#pragma unroll
            for (int g4 = 0; g4 < TC_COLS_PER_WARP / 4; ++g4) {
                if (col0 + g4 * 4 < N) {
                    uint32_t v[GR_LEVELS][4];
                    tc_load_levels4<GR_LEVELS>(trow + g4 * 4, v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        float lev[GR_LEVELS];
#pragma unroll
                        for (int L = 0; L < GR_LEVELS; ++L) lev[L] = __uint_as_float(v[L][q]);
                        long long a, b;
                        oz_levels_to_int<GR_LEVELS>(lev, a, b);
                        // lo < 2^40 before the chunk and a chunk's level 3-7 sum is < 2^56.1
                        const long long l = lo[g4 * 4 + q] + b;
                        hi[g4 * 4 + q] += a + (l >> 40);
                        lo[g4 * 4 + q] = l & ((1LL << 40) - 1);
                    }
                }
            }
            tc_fence_before_sync();
            tc_mbar_arrive(tc_smem_addr(h->bar) + 32);
            ++commits[2];
        }
        if (*(volatile int *)&h->flag) break;
    }

    if (!*(volatile int *)&h->flag) {
        // the split's exact integer sums (level 0-2 part, level 3-7 part < 2^40),
        // summed exactly over the splits and rounded once by k_gram_reduce_oz
        const int i = i0 + quarter * 32 + lane;
        long long *P = part + 2 * (long)blockIdx.z * k1 * k2;
        if (i < k1) {
#pragma unroll
            for (int q = 0; q < TC_COLS_PER_WARP; ++q) {
                const int j = j0 + col0 + q;
                if (j < k2) {
                    P[2 * (i + (long)j * k1)] = hi[q];
                    P[2 * (i + (long)j * k1) + 1] = lo[q];
                }
            }
        }
    }
    tc_release(h, tmem, mma_warp, commits, nullptr);
}

// a[i + j lda] = the exact sum over the splits of their (hi 2^40 + lo) integer
// sums, rounded once to FP64: every Gram entry is the correctly rounded value of
// the exact sum of the split operands' kept digit products, whatever the row
// split (sym: upper triangle computed, mirrored)
__global__ void k_gram_reduce_oz(int k1, int k2, int nsplit, const long long *__restrict__ part,
                                 const int *__restrict__ ev, const int *__restrict__ ew, double *__restrict__ a,
                                 int lda, int sym)
{
    const long total = (long)k1 * k2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int i = (int)(t % k1), j = (int)(t / k1);
        if (sym && i > j) continue;
        __int128 hs = 0;
        long long ls = 0;                                // nsplit < 2^23 terms below 2^40 each
        for (int q = 0; q < nsplit; ++q) {
            hs += part[2 * ((long)q * total + t)];
            ls += part[2 * ((long)q * total + t) + 1];
        }
        const __int128 z = hs * ((__int128)1 << 40) + ls;
        const double s = z == 0 ? 0.0 : oz_i128_to_double(z, ev[i] + ew[j] - OZ_SCALE_OFFSET - 56);
        a[i + (long)j * lda] = s;
        if (sym && i != j) a[j + (long)i * lda] = s;
    }
}

// a[i + j*lda] = sum_r V[r,i] W[r,j] to FP64 accuracy on the tensor cores.
// exps: device int[k1 + k2] scratch for the column scales.
extern "C" int gb_gram_tc(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *V, long ldv, const double *W,
                          long ldw, double *a_dev, int lda, int sym, int *exps)
{
    if (k1 <= 0 || k2 <= 0) return GCGE_GPU_OK;
    if (n <= 0) return gb_gram_reduce_launch(ctx, k1, k2, 0, ctx->scratch, a_dev, lda, sym);   // zeros
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_gram_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, GR_SMEM) != cudaSuccess)
            return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        attr = true;
    }
    const int ti = (k1 + TC_M - 1) / TC_M, tj = (k2 + TC_N - 1) / TC_N;
    int tiles = 0;
    for (int a = 0; a < ti; ++a)
        for (int b = 0; b < tj; ++b)
            if (!sym || a * TC_M <= b * TC_N + TC_N - 1) ++tiles;
    if (tiles < 1) tiles = 1;
    // about one CTA per SM; int64 headroom: a row adds < 2^28.2 to the level 0-2
    // sum (units of 2^-16), so a split holds at most 2^20 rows (the level 3-7 sum
    // is carried into it after every chunk)
    long nsplit = ((long)ctx->num_sms + tiles - 1) / tiles;
    const long max_split = (n + 4 * TC_KS - 1) / (4 * TC_KS);
    if (nsplit > max_split) nsplit = max_split;
    const long min_split = (n + (1L << 20) - 1) >> 20;
    if (nsplit < min_split) nsplit = min_split;
    if (nsplit < 1) nsplit = 1;
    long rps = ((n + nsplit - 1) / nsplit + TC_KS - 1) / TC_KS * TC_KS;
    nsplit = (n + rps - 1) / rps;
    if (nsplit < 1) nsplit = 1;
    int st = gb_scratch(ctx, (size_t)2 * nsplit * k1 * k2);
    if (st) return st;
    GB_LAUNCH(ctx, k_fill_int, (k1 + k2 + 127) / 128, 128, 0, exps, k1 + k2, OZ_NO_EXP);
    const int eg = ctx->num_sms * 4;
    GB_LAUNCH(ctx, k_col_exponent, eg, 256, 0, n, k1, V, ldv, exps);
    GB_LAUNCH(ctx, k_col_exponent, eg, 256, 0, n, k2, W, ldw, exps + k1);
    dim3 grid(ti, tj, (unsigned)nsplit);
    GB_PROF(ctx, GB_K_GRAM, 8.0 * n * (k1 + k2), sym ? 1.0 * n * k1 * (k1 + 1) : 2.0 * n * k1 * k2);
    const int stall = ctx->tc_stall;
    ctx->tc_stall = 0;
    long long *part = reinterpret_cast<long long *>(ctx->scratch);
    GB_LAUNCH(ctx, k_gram_tc, grid, TC_THREADS, GR_SMEM, n, k1, k2, V, ldv, W, ldw, exps, exps + k1, part, rps, sym,
              ctx->dev_err, stall);
    long rg = ((long)k1 * k2 + 255) / 256;
    if (rg > (long)ctx->num_sms * 16) rg = (long)ctx->num_sms * 16;
    GB_LAUNCH(ctx, k_gram_reduce_oz, (int)rg, 256, 0, k1, k2, (int)nsplit, part, exps, exps + k1, a_dev, lda, sym);
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- linear combination (tcgen05)
#define LC_MAX_K 4096                                // inner dimension handled by the tensor-core path
#define LC_HDR 2048                                  // tc_hdr, er, er_next, ecs
#define LC_SMEM (2 * TC_STAGE + LC_HDR + 4 * LC_MAX_K)
#define LC_OUT_LD (TC_N + 1)                         // doubles per staged output row
#define LC_CORES_PER_WARP ((TC_ACORES + TC_SPLIT_WARPS - 1) / TC_SPLIT_WARPS)
#define LC_SCALE_LOADS 48                            // row-scale loads in flight per thread
// Levels 0-7 (34 digit pairs; 8 x 64 TMEM columns): the dropped pairs (level >= 8)
// lie below 2^-55 of the scale product per term; level 7 (weight 2^-56) needs no
// exactness, levels 0-6 stay exact for OZ_EXACT_TERMS terms.
#define LC_LEVELS 8

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
    __shared__ int fs[TC_N];
    const int s = blockIdx.x, jt = blockIdx.y, j0 = jt * TC_N;
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
    for (int cc = 0; cc < TC_N / 8; ++cc) {
        const int jj = warp * (TC_N / 8) + cc, j = j0 + jj;
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
    uint32_t *out = Bd + (size_t)(jt * nst + s) * OZ_DIGITS * (TC_BPLANE / 4);
    const int n8 = lane >> 2, kp = lane & 3;
    for (int cc = 0; cc < 4; ++cc) {
        const int core = warp * 4 + cc, g = core >> 2, c = core & 3;
        const int jj = g * 8 + n8, j = j0 + jj, i = s * TC_KS + c * 8 + 2 * kp;
        unsigned long long u0 = OZ_BIAS, u1 = OZ_BIAS;
        if (j < k2) {
            if (i < k1 && (!upper || i <= j)) u0 = oz_bias(C[i + (long)j * ldc], fs[jj] + gs[i]);
            if (i + 1 < k1 && (!upper || i + 1 <= j)) u1 = oz_bias(C[i + 1 + (long)j * ldc], fs[jj] + gs[i + 1]);
        }
        const int w = (core * 128 + n8 * 16 + kp * 4) / 4;
#pragma unroll
        for (int q = 0; q < OZ_DIGITS; ++q) out[q * (TC_BPLANE / 4) + w] = oz_pack(u0, u1, q);
    }
}

// Y[r, j0 + j] = alpha sum_i X[r, i] C[i, j0 + j] + beta Y[r, j0 + j];
// grid (P, column tiles) with P <= number of SMs, TC_THREADS threads, LC_SMEM
// dynamic shared memory. Persistent: CTA b walks the 128-row tiles b, b + P, ...
// with one TMEM allocation and one barrier set; the stage counter runs across
// tiles. While the K stages of a tile run, the split warps also load the next
// tile's entries of the same stage and fold their exponents into that tile's row
// scales (shared-memory atomicMax) one stage later, when the loads have landed,
// so only the first tile has a separate scale pass and every later tile's X is
// already in L2 when it is split. The drain
// writes Y directly. MULTI: the inner dimension is longer than one exact
// accumulation (k1 > OZ_EXACT_TERMS) and the drained chunks are summed in
// registers; the single-chunk form holds no FP64 accumulators while it splits.
template <bool MULTI>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_lincomb_tc(int n, int k1, int k2, const double *__restrict__ X, long ldx, const uint4 *__restrict__ Bd,
             const int *__restrict__ g_in, const int *__restrict__ ec, double alpha, double beta,
             double *__restrict__ Y, long ldy, int nst, int *__restrict__ err, int stall)
{
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint8_t *sm = tc_smem;
    if (*(volatile int *)err) return;                    // an earlier launch timed out: do nothing
    tc_hdr *h = (tc_hdr *)(sm + 2 * TC_STAGE);
    int *er = (int *)(sm + 2 * TC_STAGE + 64);           // [TC_M] row scales of X 2^g, this tile
    int *er_next = er + TC_M;                            // [TC_M] the same for the next tile
    int *ecs = er_next + TC_M;                           // [TC_N] column scales of 2^-g C
    int *gs = (int *)(sm + 2 * TC_STAGE + LC_HDR);       // [k1] inner-dimension scales g
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int jt = blockIdx.y, j0 = jt * TC_N;
    const int N = min(TC_N, (k2 - j0 + 15) & ~15);
    const long ntiles = ((long)n + TC_M - 1) / TC_M;
    // one exact accumulation over all of K when it is short enough
    const int chunk_stages = k1 <= OZ_EXACT_TERMS ? nst : TC_CHUNK_STAGES;

    tc_setup(h);
    for (int i = tid; i < k1; i += TC_THREADS) gs[i] = g_in[i];
    if (tid < TC_N) ecs[tid] = j0 + tid < k2 ? ec[j0 + tid] : OZ_NO_EXP;
    if (tid < TC_M) er_next[tid] = OZ_NO_EXP;
    __syncthreads();
    // row scales of the first tile: 4 threads per row, up to LC_SCALE_LOADS
    // independent loads of the high words (sign, exponent) in flight per thread
    {
        const int rr = tid >> 2, t4 = tid & 3;
        const long r = (long)blockIdx.x * TC_M + rr;
        const bool rin = r < n;
        const unsigned *xh = reinterpret_cast<const unsigned *>(X + (rin ? r : 0) * ldx) + 1;
        int e = OZ_NO_EXP;
        for (int i0 = t4; i0 < k1; i0 += 4 * LC_SCALE_LOADS) {
            unsigned w[LC_SCALE_LOADS];
#pragma unroll
            for (int j = 0; j < LC_SCALE_LOADS; ++j) {
                const int i = i0 + 4 * j;
                w[j] = (rin && i < k1) ? __ldg(xh + 2 * (long)i) : 0u;
            }
#pragma unroll
            for (int j = 0; j < LC_SCALE_LOADS; ++j) {
                const int i = i0 + 4 * j;
                const int ex = (int)((w[j] >> 20) & 0x7ff);
                const int gi = i < k1 ? gs[i] : OZ_NO_EXP;
                if (ex && gi != OZ_NO_EXP) e = max(e, ex - 1022 + gi);
            }
        }
        e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));
        e = max(e, __shfl_xor_sync(0xffffffffu, e, 2));
        if (t4 == 0) er[rr] = e;
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const uint32_t tmem = h->tmem, sbase = tc_smem_addr(sm);
    const bool mma_warp = warp == TC_SPLIT_WARPS;
    const int quarter = warp & 3, col0 = (warp >> 2) * TC_COLS_PER_WARP;
    const int my_row = quarter * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16) + col0;
    // alpha = +-1, beta = 0: the output is the drained value with its sign bit
    // flipped or not, an integer operation (the FP64 pipe runs at 1/64 rate)
    const bool plain = beta == 0.0 && (alpha == 1.0 || alpha == -1.0);
    const unsigned long long sflip = alpha == -1.0 ? 0x8000000000000000ull : 0ull;
    int commits[3] = {0, 0, 0};
    int copies[2] = {0, 0};                              // bulk copies per buffer (thread 0)

    // split-warp geometry: core q = warp + 15 cc (A cores only); lane (r8, kp):
    // row 8g + r8, entries 8c + 2 kp and 8c + 2 kp + 1
    const int r8 = lane >> 2, kp = lane & 3;
    double xv[LC_CORES_PER_WARP][2];
    auto load_stage = [&](long row0, int s) {
        const int ib = s * TC_KS + 2 * kp;
#pragma unroll
        for (int cc = 0; cc < LC_CORES_PER_WARP; ++cc) {
            const int q = warp + TC_SPLIT_WARPS * cc;
            const long r = row0 + 8 * (q >> 2) + r8;
            const int i = ib + 8 * (q & 3);
            const bool in = q < TC_ACORES && r < n;
            xv[cc][0] = (in && i < k1) ? X[r * ldx + i] : 0.0;
            xv[cc][1] = (in && i + 1 < k1) ? X[r * ldx + i + 1] : 0.0;
        }
    };
    if (!mma_warp) load_stage((long)blockIdx.x * TC_M, 0);
    // high words (sign, exponent) of the next tile's entries of one stage, in flight
    unsigned pw[LC_CORES_PER_WARP][2];
    int pw_stage = -1;
    auto fold_scales = [&](int ps) {
        const int ib = ps * TC_KS + 2 * kp;
#pragma unroll
        for (int cc = 0; cc < LC_CORES_PER_WARP; ++cc) {
            const int q = warp + TC_SPLIT_WARPS * cc;
            if (q < TC_ACORES) {
                const int i = ib + 8 * (q & 3);
                int e = OZ_NO_EXP;
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int ex = (int)((pw[cc][u] >> 20) & 0x7ff);
                    const int gi = i + u < k1 ? gs[i + u] : OZ_NO_EXP;
                    if (ex && gi != OZ_NO_EXP) e = max(e, ex - 1022 + gi);
                }
                e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));
                e = max(e, __shfl_xor_sync(0xffffffffu, e, 2));
                if (kp == 0 && e > OZ_NO_EXP) atomicMax(er_next + 8 * (q >> 2) + r8, e);
            }
        }
    };

    int gsc = 0;                                         // stages issued by this CTA, over all tiles
    bool stop = false;
    for (long t = blockIdx.x; t < ntiles && !stop; t += gridDim.x) {
        const long row0 = t * TC_M, nrow0 = row0 + (long)gridDim.x * TC_M;
        const bool has_next = t + gridDim.x < ntiles;
        const int my_e = er[my_row];
        double acc[MULTI ? TC_COLS_PER_WARP : 1];
#pragma unroll
        for (int q = 0; q < (MULTI ? TC_COLS_PER_WARP : 1); ++q) acc[q] = 0.0;
        for (int s = 0; s < nst; ++s, ++gsc) {
            const int buf = gsc & 1, cs = s % chunk_stages;
            const bool chunk_end = cs == chunk_stages - 1 || s == nst - 1;
            if (mma_warp) {
                if (lane == 0) tc_issue_stage<LC_LEVELS, true>(h, sbase, tmem, N, gsc, cs, commits, err, stall);
                __syncwarp();
            } else {
                if (gsc >= 2 && !tc_mbar_wait(tc_smem_addr(h->bar) + 16 + 8 * buf, ((gsc >> 1) - 1) & 1,
                                              TC_WAIT_NS))
                    tc_fail(h, err);
                uint8_t *A = sm + buf * TC_STAGE;
                uint8_t *B = A + OZ_DIGITS * TC_APLANE;
                const uint32_t full = tc_smem_addr(h->bar) + 8 * buf;
                // the pre-split C planes of this stage: one bulk copy, completing on copied[buf]
                if (tid == 0) {
                    const uint32_t copied = tc_smem_addr(h->bar) + 40 + 8 * buf;
                    tc_mbar_arrive_expect_tx(copied, OZ_DIGITS * TC_BPLANE);
                    tc_bulk_g2s(tc_smem_addr(B), Bd + (size_t)(jt * nst + s) * (OZ_DIGITS * TC_BPLANE / 16),
                                OZ_DIGITS * TC_BPLANE, copied);
                    ++copies[buf];
                }
                const int ib = s * TC_KS + 2 * kp;
#pragma unroll
                for (int cc = 0; cc < LC_CORES_PER_WARP; ++cc) {
                    const int q = warp + TC_SPLIT_WARPS * cc;
                    if (q < TC_ACORES) {
                        const int i = ib + 8 * (q & 3);
                        const int e = er[8 * (q >> 2) + r8];
                        // a zero row of C (g = OZ_NO_EXP) contributes nothing: its digits stay zero
                        const int g0 = i < k1 ? gs[i] : OZ_NO_EXP, g1 = i + 1 < k1 ? gs[i + 1] : OZ_NO_EXP;
                        const unsigned long long u0 = g0 != OZ_NO_EXP ? oz_bias(xv[cc][0], e - g0) : OZ_BIAS;
                        const unsigned long long u1 = g1 != OZ_NO_EXP ? oz_bias(xv[cc][1], e - g1) : OZ_BIAS;
                        uint32_t *dst = (uint32_t *)(A + q * 128 + r8 * 16 + kp * 4);
#pragma unroll
                        for (int p = 0; p < OZ_DIGITS; ++p) dst[p * (TC_APLANE / 4)] = oz_pack(u0, u1, p);
                    }
                }
                tc_fence_async_smem();
                tc_mbar_arrive(full);
                // in flight while the MMAs run: the next stage's values (or the next
                // tile's first stage), and the next tile's entries of this stage for its scales
                if (s + 1 < nst) load_stage(row0, s + 1);
                else if (has_next) load_stage(nrow0, 0);
                // the next tile's high words of the previous stage arrived while this
                // stage was split: fold them into its row scales now, then issue this
                // stage's (consumed one stage later, so no load latency is waited on)
                if (pw_stage >= 0) fold_scales(pw_stage);
                pw_stage = -1;
                if (has_next) {
#pragma unroll
                    for (int cc = 0; cc < LC_CORES_PER_WARP; ++cc) {
                        const int q = warp + TC_SPLIT_WARPS * cc;
                        const long r = nrow0 + 8 * (q >> 2) + r8;
                        const int i = ib + 8 * (q & 3);
                        const bool in = q < TC_ACORES && r < n;
                        const unsigned *xh = reinterpret_cast<const unsigned *>(X + (in ? r : 0) * ldx + i) + 1;
                        pw[cc][0] = (in && i < k1) ? __ldg(xh) : 0u;
                        pw[cc][1] = (in && i + 1 < k1) ? __ldg(xh + 2) : 0u;
                    }
                    pw_stage = s;
                }
            }
            if (chunk_end) {
                if (!tc_wait_chunk(h, gsc, err)) {
                    stop = true;
                    break;
                }
                const bool first = s < chunk_stages, last = s == nst - 1;
                const long r = row0 + my_row;
#pragma unroll
                for (int g4 = 0; g4 < TC_COLS_PER_WARP / 4; ++g4) {
                    if (col0 + g4 * 4 < N) {
                        uint32_t v[LC_LEVELS][4];
                        tc_load_levels4<LC_LEVELS>(trow + g4 * 4, v);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            float lev[LC_LEVELS];
#pragma unroll
                            for (int L = 0; L < LC_LEVELS; ++L) lev[L] = __uint_as_float(v[L][q]);
                            long long a, b;
                            oz_levels_to_int<LC_LEVELS>(lev, a, b);
                            const double d =
                                oz_to_double40(a, b, my_e + ecs[col0 + g4 * 4 + q] - OZ_SCALE_OFFSET);
                            double v2 = d;
                            if (MULTI) {
                                acc[g4 * 4 + q] = first ? d : acc[g4 * 4 + q] + d;
                                v2 = acc[g4 * 4 + q];
                            }
                            const int j = j0 + col0 + g4 * 4 + q;
                            if (last && r < n && j < k2) {
                                double *y = Y + r * ldy + j;
                                if (plain)
                                    *y = __longlong_as_double(__double_as_longlong(v2) ^ (long long)sflip);
                                else
                                    *y = fma(beta, *y, alpha * v2);
                            }
                        }
                    }
                }
                tc_fence_before_sync();
                tc_mbar_arrive(tc_smem_addr(h->bar) + 32);
                ++commits[2];
            }
            if (*(volatile int *)&h->flag) {
                stop = true;
                break;
            }
        }
        // tile end: fold the last stage's words (they arrived during the drain); then
        // every scale atomic of the next tile is done; er <- er_next
        if (!mma_warp && pw_stage >= 0) {
            __syncwarp();
            fold_scales(pw_stage);
            pw_stage = -1;
        }
        __syncthreads();
        if (tid < TC_M) {
            er[tid] = er_next[tid];
            er_next[tid] = OZ_NO_EXP;
        }
        __syncthreads();
        if (*(volatile int *)&h->flag) stop = true;
    }
    tc_release(h, tmem, mma_warp, commits, copies);
}

extern "C" int gb_lincomb_tc_ok(int k1) { return k1 <= LC_MAX_K; }
// Y may overlap X's columns (the same rows, the same leading dimension) when one
// column tile covers the output: a CTA reads every entry of its row tile before
// its drain writes that tile's rows, and walks only its own tiles (the
// next-tile prefetch and scale pass included)
extern "C" int gb_lincomb_tc_inplace_ok(int k1, int k2) { return k1 <= LC_MAX_K && k2 <= TC_N; }

// Y = alpha X C + beta Y (C: k1 x k2 column-major on the device, upper: only
// i <= j of C is used) to FP64 accuracy on the tensor cores.
extern "C" int gb_lincomb_tc(gcge_gpu_ctx *ctx, int n, int k1, int k2, const double *X, long ldx, const double *C,
                             int ldc, double alpha, double beta, double *Y, long ldy, int upper)
{
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_lincomb_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, LC_SMEM) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_lincomb_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, LC_SMEM) !=
                cudaSuccess)
            return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        attr = true;
    }
    const int nst = (k1 + TC_KS - 1) / TC_KS, jtiles = (k2 + TC_N - 1) / TC_N;
    const size_t bd_bytes = (size_t)jtiles * nst * OZ_DIGITS * TC_BPLANE;
    int st = gb_ozbuf(ctx, bd_bytes);
    if (!st) st = gb_iscratch(ctx, (size_t)k1 + k2);
    if (st) return st;
    uint32_t *Bd = (uint32_t *)ctx->ozbuf;
    int *g = ctx->iscratch, *ec = ctx->iscratch + k1;
    GB_LAUNCH(ctx, k_lc_coef_split, dim3(nst, jtiles), 256, 0, k1, k2, C, ldc, upper, nst, g, ec, Bd);
    GB_PROF(ctx, GB_K_LINCOMB, 8.0 * n * k1 + (beta != 0.0 ? 16.0 : 8.0) * n * k2,
            upper ? 1.0 * n * k1 * (k2 + 1) : 2.0 * n * k1 * k2);
    const long ntiles = ((long)n + TC_M - 1) / TC_M;
    long P = ctx->num_sms / jtiles;
    if (P < 1) P = 1;
    if (P > ntiles) P = ntiles;
    const int stall = ctx->tc_stall;
    ctx->tc_stall = 0;
    if (k1 > OZ_EXACT_TERMS)
        GB_LAUNCH(ctx, k_lincomb_tc<true>, dim3((unsigned)P, jtiles), TC_THREADS, LC_SMEM, n, k1, k2, X, ldx,
                  (const uint4 *)Bd, g, ec, alpha, beta, Y, ldy, nst, ctx->dev_err, stall);
    else
        GB_LAUNCH(ctx, k_lincomb_tc<false>, dim3((unsigned)P, jtiles), TC_THREADS, LC_SMEM, n, k1, k2, X, ldx,
                  (const uint4 *)Bd, g, ec, alpha, beta, Y, ldy, nst, ctx->dev_err, stall);
    return GCGE_GPU_OK;
}
