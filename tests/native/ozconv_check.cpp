// CPU check of the 64-bit FP64 conversion of the tensor-core linear combination
// (oz_to_double40) against the general 128-bit form (oz_to_double<40>): both must
// give the same bits for every combination of eight levels the drain can produce.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "gb_ozconv.h"

static unsigned long long bits(double d)
{
    unsigned long long u;
    memcpy(&u, &d, sizeof u);
    return u;
}

static void combine(const long long *v, long long &hi, long long &lo)
{
    hi = (v[0] << 16) + (v[1] << 8) + v[2];
    lo = (v[3] << 32) + (v[4] << 24) + (v[5] << 16) + (v[6] << 8) + v[7];
}

int main(int argc, char **argv)
{
    const long cases = argc > 1 ? atol(argv[1]) : 2000000;
    std::mt19937_64 rng(20261203);
    long bad = 0, tested = 0;
    auto check = [&](const long long *v, int s) {
        long long hi, lo;
        combine(v, hi, lo);
        const double a = oz_to_double<40>(hi, lo, s), b = oz_to_double40(hi, lo, s);
        ++tested;
        if (bits(a) != bits(b)) {
            if (bad < 10)
                printf("mismatch v=[%lld %lld %lld %lld %lld %lld %lld %lld] s=%d: %.17g vs %.17g\n", v[0], v[1], v[2],
                       v[3], v[4], v[5], v[6], v[7], s, a, b);
            ++bad;
        }
    };
    const long long LIM = 1LL << 24;
    long long v[8];
    for (long c = 0; c < cases; ++c) {
        // magnitudes from tiny to the exact-accumulation limit, independent per level
        for (int L = 0; L < 8; ++L) {
            const int mb = (int)(rng() % 26);
            const long long m = mb ? (long long)(rng() % (1ULL << mb)) : 0;
            v[L] = (rng() & 1) ? -m : m;
            if (v[L] > LIM) v[L] = LIM;
            if (v[L] < -LIM) v[L] = -LIM;
        }
        // leading levels zero now and then (small results, cancellation)
        const int z = (int)(rng() % 8);
        for (int L = 0; L < z && (c & 3) == 0; ++L) v[L] = 0;
        check(v, (int)(rng() % 200) - 100);
    }
    // ties and carries: a level pattern that puts exactly half an ulp below the
    // 53-bit point, in both signs, for every shift of the leading level
    for (int top = 0; top < 25; ++top)
        for (int sg = -1; sg <= 1; sg += 2)
            for (int t = 0; t < 4; ++t) {
                memset(v, 0, sizeof v);
                v[0] = sg * (1LL << top);
                v[7] = sg * (t == 0 ? 1 : t == 1 ? -1 : t == 2 ? 128 : -128);
                v[5] = sg * (t & 1);
                check(v, 0);
                v[0] = sg * ((1LL << top) - 1);
                check(v, 3);
            }
    // exponent range edges (the FP64 fallback)
    for (int s = -1100; s <= 1100; s += 7) {
        for (int L = 0; L < 8; ++L) v[L] = (long long)(rng() % (1ULL << 20)) - (1LL << 19);
        check(v, s);
    }
    printf("tested %ld mismatches %ld\n", tested, bad);
    return bad != 0;
}
