// Double-float ("df64") arithmetic for the FP64 tile pass.
//
// GB300's CUDA cores run FP64 at a small fraction of their FP32 rate, and the
// FP64 tile pass is bound by that FP64 pipe (two FP64 instructions per
// amplitude per arithmetic gate).  A df64 value is an unevaluated sum hi + lo of
// two FP32 numbers (|lo| below one unit in the last place of hi), 48 significand
// bits, with every operation on the FP32 pipe.  The algorithms are the published
// double-float ones (T. J. Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971; Y. Hida, X. S. Li, D. H. Bailey,
// "Algorithms for quad-double precision floating point arithmetic", ARITH-15,
// 2001: two-sum, fast two-sum, FMA-based two-product, the "sloppy" addition).
//
// Conversions between IEEE double (the state's storage format) and df64 use
// integer bit operations only, so no instruction of a converted pass runs on the
// FP64 pipe: the high part is the double's sign, exponent and top 23 fraction
// bits, the low part the remaining 29 fraction bits converted to FP32 and scaled
// by a power of two; back, the low part is aligned to the double's 52-bit
// significand grid and added as an integer.  Magnitudes below 2^-126 convert to
// zero, and below about 2^-102 the low part is an FP32 subnormal with fewer
// bits; amplitudes of a normalised state stay far above both in practice.
//
// Written as host and device code so the CPU test suite checks it.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

#ifndef __CUDACC__
#define SQ_HD inline
#else
#define SQ_HD __host__ __device__ __forceinline__
#endif

namespace sqk {

struct df64 {
    float hi, lo;
};

SQ_HD uint32_t df_fbits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
SQ_HD float df_bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}
SQ_HD uint64_t df_dbits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
#endif
}
SQ_HD double df_bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    std::memcpy(&x, &u, 8);
    return x;
#endif
}
SQ_HD float df_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
SQ_HD int df_clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// IEEE double -> df64 (integer operations only)
SQ_HD df64 df_from_double(double d) {
    const uint64_t b = df_dbits(d);
    const uint32_t sign = (uint32_t)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7FFu);  // biased double exponent
    df64 r;
    if (e <= 896) {  // below the FP32 normal range (and zero)
        r.hi = df_bitsf(sign);
        r.lo = df_bitsf(sign);
        return r;
    }
    const uint64_t m = b & 0xFFFFFFFFFFFFFull;
    r.hi = df_bitsf(sign | ((uint32_t)(e - 896) << 23) | (uint32_t)(m >> 29));
    // low 29 fraction bits, worth m29 * 2^(e - 1075): scaled by 2^(e - 975) (an FP32
    // normal for every e here) and then by 2^-100, both exact until the result
    // itself leaves the normal range
    const uint32_t m29 = (uint32_t)(m & 0x1FFFFFFFu);
    const float scale = df_bitsf((uint32_t)(e - 848) << 23);
    r.lo = df_bitsf(df_fbits(((float)m29 * scale) * 7.888609052210118e-31f) | sign);  // 2^-100
    return r;
}

// df64 -> IEEE double, rounded (integer operations only)
SQ_HD double df_to_double(df64 a) {
    const uint32_t hb = df_fbits(a.hi), lb = df_fbits(a.lo);
    const int eh = (int)((hb >> 23) & 0xFFu);
    if (eh == 0) return df_bitsd((uint64_t)(hb >> 31) << 63);  // zero (FP32 subnormals do not occur)
    // hi = MH 2^(eh-150) = (MH << 29) 2^(eh-179): work on the grid 2^(eh-179)
    int64_t M = (int64_t)((uint64_t)((hb & 0x7FFFFFu) | 0x800000u) << 29);
    int el = (int)((lb >> 23) & 0xFFu);
    if ((lb & 0x7FFFFFFFu) != 0u) {
        // lo = ML 2^(el-150); a subnormal low part has no implicit bit and el = 1
        const uint64_t ML = el ? (uint64_t)((lb & 0x7FFFFFu) | 0x800000u) : (uint64_t)(lb & 0x7FFFFFu);
        if (!el) el = 1;
        const int sh = el - eh + 29;                                  // lo on the grid: ML 2^sh
        uint64_t dlt;
        if (sh >= 0)
            dlt = sh < 34 ? ML << sh : 0ull;  // |lo| < 2^-5 |hi| always holds for df64 values
        else
            dlt = sh > -40 ? (ML + (1ull << (-sh - 1))) >> (-sh) : 0ull;
        if ((lb ^ hb) >> 31) M -= (int64_t)dlt;
        else M += (int64_t)dlt;
    }
    // M is positive and within a factor 2 of 2^52.5: renormalise to [2^52, 2^53)
    int E = eh + 896;  // biased double exponent of the grid's 2^52 position
    uint64_t U = (uint64_t)M;
    const int lz = df_clz64(U);
    if (lz < 11) {  // >= 2^53: shift right, rounding half up
        const int s = 11 - lz;
        U = (U + (1ull << (s - 1))) >> s;
        E += s;
        if (U >> 53) {
            U >>= 1;
            E += 1;
        }
    } else if (lz > 11) {
        const int s = lz - 11;
        U <<= s;
        E -= s;
    }
    return df_bitsd(((uint64_t)(hb >> 31) << 63) | ((uint64_t)E << 52) | (U & 0xFFFFFFFFFFFFFull));
}

// exact sum of two floats as (s, e): s = fl(a + b), s + e = a + b (Knuth / Dekker two-sum)
SQ_HD void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// the same when |a| >= |b| (fast two-sum)
SQ_HD void fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}

SQ_HD df64 df_add(df64 a, df64 b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    df64 r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
SQ_HD df64 df_neg(df64 a) { return df64{-a.hi, -a.lo}; }
SQ_HD df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }
// product with the FMA-based two-product of the high parts
SQ_HD df64 df_mul(df64 a, df64 b) {
    const float p = a.hi * b.hi;
    float e = df_fma(a.hi, b.hi, -p);
    e = df_fma(a.hi, b.lo, e);
    e = df_fma(a.lo, b.hi, e);
    df64 r;
    fast_two_sum(p, e, r.hi, r.lo);
    return r;
}
// a * b + c
SQ_HD df64 df_fmadd(df64 a, df64 b, df64 c) {
    const float p = a.hi * b.hi;
    float pe = df_fma(a.hi, b.hi, -p);
    pe = df_fma(a.hi, b.lo, pe);
    pe = df_fma(a.lo, b.hi, pe);
    float s, e;
    two_sum(p, c.hi, s, e);
    e += pe + c.lo;
    df64 r;
    fast_two_sum(s, e, r.hi, r.lo);
    return r;
}
// a with its sign flipped when f
SQ_HD df64 df_neg_if(df64 a, bool f) {
    const uint32_t m = (uint32_t)f << 31;
    return df64{df_bitsf(df_fbits(a.hi) ^ m), df_bitsf(df_fbits(a.lo) ^ m)};
}
SQ_HD df64 operator+(df64 a, df64 b) { return df_add(a, b); }
SQ_HD df64 operator-(df64 a, df64 b) { return df_sub(a, b); }
SQ_HD df64 operator-(df64 a) { return df_neg(a); }
SQ_HD df64 operator*(df64 a, df64 b) { return df_mul(a, b); }


// a df64 constant from a double computed on the host (exact split, no flush)
inline df64 df_const_host(double d) {
    df64 r;
    r.hi = (float)d;
    r.lo = (float)(d - (double)r.hi);
    return r;
}

}  // namespace sqk
