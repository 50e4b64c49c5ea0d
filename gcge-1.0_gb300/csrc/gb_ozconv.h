// gb_ozconv.h -- exact integer -> FP64 conversions of the error-free digit
// splitting (host and device code, no intrinsics beyond count-leading-zeros and
// a bit cast, so that the same functions compile into a CPU check).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define OZ_HD __host__ __device__ __forceinline__
#else
#define OZ_HD inline
#endif

OZ_HD int oz_clz64(unsigned long long x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

OZ_HD double oz_bits_to_double(unsigned long long u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, sizeof d);
    return d;
#endif
}

// (hi 2^SH + lo) 2^(s - 16 - SH) rounded once to nearest-even, s = e + f -
// OZ_SCALE_OFFSET: hi holds levels 0-2 in units of 2^-16, lo the lower levels in
// units of 2^-(16 + SH) (SH = 32 for levels 3-6, 40 for levels 3-7). General
// 128-bit form (any hi, lo).
template <int SH>
OZ_HD double oz_to_double(long long hi, long long lo, int s)
{
    __int128 z = ((__int128)hi << SH) + (__int128)lo;
    if (z == 0) return 0.0;
    unsigned long long sign = 0;
    if (z < 0) {
        sign = 1ull << 63;
        z = -z;
    }
    const unsigned __int128 u = (unsigned __int128)z;
    const unsigned long long zh = (unsigned long long)(u >> 64), zl = (unsigned long long)u;
    const int nb = zh ? 128 - oz_clz64(zh) : 64 - oz_clz64(zl);
    int E = nb - 1 + s - 16 - SH;
    unsigned long long m;
    if (nb <= 53) {
        m = zl << (53 - nb);
    } else {
        const int sh = nb - 53;
        const unsigned __int128 q = u >> sh;
        const unsigned __int128 rem = u - (q << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        m = (unsigned long long)q;
        if (rem > half || (rem == half && (m & 1))) ++m;
        if (m >> 53) {
            m >>= 1;
            ++E;
        }
    }
    if (E < -1022 || E > 1023)                     // outside the normal range: scale in FP64
        return ldexp((double)hi, s - 16) + ldexp((double)lo, s - 16 - SH);
    return oz_bits_to_double(sign | ((unsigned long long)(E + 1023) << 52) | (m & ((1ull << 52) - 1)));
}

// z 2^e0 rounded once to nearest-even, z any 128-bit integer (the exact sum of a
// Gram entry's split partials, hi 2^40 + lo summed over the splits)
OZ_HD double oz_i128_to_double(__int128 z, int e0)
{
    if (z == 0) return 0.0;
    unsigned long long sign = 0;
    if (z < 0) {
        sign = 1ull << 63;
        z = -z;
    }
    const unsigned __int128 u = (unsigned __int128)z;
    const unsigned long long zh = (unsigned long long)(u >> 64), zl = (unsigned long long)u;
    const int nb = zh ? 128 - oz_clz64(zh) : 64 - oz_clz64(zl);
    int E = nb - 1 + e0;
    unsigned long long m;
    if (nb <= 53) {
        m = zl << (53 - nb);
    } else {
        const int sh = nb - 53;
        const unsigned __int128 q = u >> sh;
        const unsigned __int128 rem = u - (q << sh);
        const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        m = (unsigned long long)q;
        if (rem > half || (rem == half && (m & 1))) ++m;
        if (m >> 53) {
            m >>= 1;
            ++E;
        }
    }
    if (E < -1022 || E > 1023) {                   // outside the normal range: scale in FP64
        const double mag = ldexp((double)zh, e0 + 64) + ldexp((double)zl, e0);
        return sign ? -mag : mag;
    }
    return oz_bits_to_double(sign | ((unsigned long long)(E + 1023) << 52) | (m & ((1ull << 52) - 1)));
}

// The same value for SH = 40 in 64-bit arithmetic, for |hi| < 2^41 and |lo| < 2^62
// (eight levels of at most 2^24 each). z = hi 2^40 + lo = T 2^18 + R with T =
// floor(z / 2^18) (|T| < 2^63) and 0 <= R < 2^18; |z| is carried as U 2^e where
// U is exact (|z| < 2^63) or U keeps at least 55 bits and the discarded bits are
// folded into its lowest bit (round to odd), so that rounding U once to 53 bits
// (nearest-even) gives the correctly rounded |z| -- the result of the general
// form bit for bit.
OZ_HD double oz_to_double40(long long hi, long long lo, int s)
{
    const long long T = hi * (1LL << 22) + (lo >> 18);
    const unsigned long long R = (unsigned long long)(lo & 0x3ffffLL);
    if (T == 0 && R == 0) return 0.0;
    unsigned long long sign = 0, Tm = (unsigned long long)T, Rm = R;
    if (T < 0) {
        sign = 1ull << 63;
        Tm = R ? (unsigned long long)(-(T + 1)) : (unsigned long long)(-T);
        Rm = R ? (1ull << 18) - R : 0;
    }
    unsigned long long U;
    int e;
    if (Tm < (1ull << 45)) {
        U = (Tm << 18) | Rm;
        e = 0;
    } else if (Tm < (1ull << 55)) {
        U = (Tm << 9) | (Rm >> 9) | (unsigned long long)((Rm & 0x1ffull) != 0);
        e = 9;
    } else {
        U = Tm | (unsigned long long)(Rm != 0);
        e = 18;
    }
    const int nb = 64 - oz_clz64(U);
    int E = nb - 1 + e + s - 56;
    unsigned long long m;
    if (nb <= 53) {
        m = U << (53 - nb);
    } else {
        const int sh = nb - 53;
        m = U >> sh;
        const unsigned long long rem = U & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (m & 1))) ++m;
        if (m >> 53) {
            m >>= 1;
            ++E;
        }
    }
    if (E < -1022 || E > 1023)
        return ldexp((double)hi, s - 16) + ldexp((double)lo, s - 56);
    return oz_bits_to_double(sign | ((unsigned long long)(E + 1023) << 52) | (m & ((1ull << 52) - 1)));
}
