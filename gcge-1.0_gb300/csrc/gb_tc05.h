// gb_tc05.h -- inline-PTX primitives for the 5th-generation tensor cores
// (tcgen05: TMEM accumulators, shared-memory operand descriptors, mbarriers)
// and the error-free FP64 digit splitting shared by the tensor-core kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// ---------------------------------------------------------------- addresses, fences
__device__ __forceinline__ uint32_t tc_smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void tc_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ uint64_t tc_globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------- TMEM
// allocation by one whole warp; the TMEM address is written to smem[dst]
__device__ __forceinline__ void tc_tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 32 lanes x 8 consecutive 32-bit columns (lane = warp's quarter of the 128 lanes);
// the values may be used only after tc_tmem_wait8 on the same registers
__device__ __forceinline__ void tc_tmem_ld8(uint32_t taddr, uint32_t r[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tc_tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// ties registers loaded by tc_tmem_ld8 to a point after tc_tmem_wait_ld
__device__ __forceinline__ void tc_reg_fence8(uint32_t r[8])
{
    asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]));
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void tc_mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool tc_mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tc_mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// arrival that also expects `bytes` of asynchronous copies to complete on the barrier
__device__ __forceinline__ void tc_mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16),
// completing its bytes on the mbarrier
__device__ __forceinline__ void tc_bulk_g2s(uint32_t dst_smem, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     dst_smem),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// barrier over the first `count` threads of the CTA (named barrier `id`, 1..15)
__device__ __forceinline__ void tc_bar_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// bounded wait for the phase of the given parity; false after limit_ns
__device__ __forceinline__ bool tc_mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns)
{
    if (tc_mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = tc_globaltimer();
    while (!tc_mbar_try_wait(bar, parity))
        if (tc_globaltimer() - t0 > limit_ns) return false;
    return true;
}

// ---------------------------------------------------------------- MMA
// shared-memory matrix descriptor, no swizzle: 8-row x 16-byte core matrices of
// 128 contiguous bytes; lbo = byte distance of core matrices adjacent in K,
// sbo = byte distance of core matrices adjacent in M (or N)
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}
// instruction descriptor of kind::f16: bf16 x bf16 -> f32, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// the same for f16 x f16 -> f32
__host__ __device__ constexpr uint32_t tc_idesc_f16(int M, int N)
{
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D[tmem] (+)= A[smem] * B[smem]^T (kind::f16, types from idesc), issued by one thread
__device__ __forceinline__ void tc_mma_kf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
                 : "memory");
}
// mbarrier arrive once all tcgen05 operations issued so far by this thread are done
__device__ __forceinline__ void tc_mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// ---------------------------------------------------------------- error-free digit splitting
// An FP64 entry x of a row (or column) with scale 2^e (|x| < 2^e over the row)
// is the integer T = x 2^(53 - e) rounded to nearest, |T| <= 2^53, i.e. exact to
// half a unit of 2^(e - 53). With the bias B = 0x80808080808080, U = T + B lies
// in [0, 2^56) and its seven bytes b_0 (least significant) .. b_6 give balanced
// digits d_p = b_(6-p) - 128:
//   x = sum_p d_p 2^(-8p) 2^(e - 5),   p = 0 (most significant) .. 6,
// with d_0 in [-32, 32] and d_1 .. d_6 in [-128, 127]. Only integer operations
// touch x; every digit is exact in f16 (and bf16).
//
// Exact accumulation bound: the digit products of level L = p + q are at most
// 2^12 for the two pairs with p = 0 or q = 0 and 2^14 for the others, so a
// level sums to at most 2^13 + 5 * 2^14 per term (L = 6) and stays below 2^24
// -- an exact FP32 integer -- for up to OZ_EXACT_TERMS terms.
#define OZ_DIGITS 7
#define OZ_NO_EXP (-2000)          // scale of an all-zero row or column
#define OZ_BIAS 0x80808080808080ULL
#define OZ_EXACT_TERMS 186
#define OZ_SCALE_OFFSET 10         // a digit product of level 0 carries 2^(e + f - 10)

__device__ __forceinline__ unsigned long long oz_bias(double x, int e)
{
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    long long T = 0;
    const int r = e + 1022 - ex;                          // T = mant 2^-r, r >= 0
    if (ex && r < 60) {
        const long long mant = (b & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
        T = (mant + ((1LL << r) >> 1)) >> r;
        if (b < 0) T = -T;
    }
    return (unsigned long long)T + OZ_BIAS;
}
// exponent contribution of one entry: |x| < 2^(ex - 1022); OZ_NO_EXP for 0 and subnormals
__device__ __forceinline__ int oz_exponent(double x)
{
    const int ex = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
    return ex ? ex - 1022 : OZ_NO_EXP;
}
// digit p of two biased values as one f16x2 word (u0 in the low half): the
// bytes b are placed as 0x64bb = 1024 + b and 1152 is subtracted, both exact
__device__ __forceinline__ uint32_t oz_pack(unsigned long long u0, unsigned long long u1, int p)
{
    const int byte = 6 - p, b = byte & 3;
    const uint32_t w0 = byte < 4 ? (uint32_t)u0 : (uint32_t)(u0 >> 32);
    const uint32_t w1 = byte < 4 ? (uint32_t)u1 : (uint32_t)(u1 >> 32);
    const uint32_t t = __byte_perm(w0, w1, (uint32_t)(b | (b << 4) | ((b + 4) << 8) | ((b + 4) << 12)));
    const uint32_t h = (t & 0x00FF00FFu) | 0x64006400u;
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(h), "r"(0x64806480u));
    return r;
}

#include "gb_ozconv.h"

// levels (exact FP32 integers) -> hi (levels 0-2, units 2^-16) and lo (levels
// 3 .. LEVELS-1 in units of the lowest level) of one output
template <int LEVELS>
__device__ __forceinline__ void oz_levels_to_int(const float *v, long long &hi, long long &lo)
{
    hi = ((long long)__float2int_rn(v[0]) << 16) + ((long long)__float2int_rn(v[1]) << 8) +
         (long long)__float2int_rn(v[2]);
    lo = 0;
#pragma unroll
    for (int L = 3; L < LEVELS; ++L) lo += (long long)__float2int_rn(v[L]) << (8 * (LEVELS - 1 - L));
}
