// Float-float ("double-FP32") arithmetic for the FP64 form's pair kernel.
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so the pair geometry, the
// overlap velocities and the gas-exchange terms of the FP64 form are carried
// as unevaluated sums h + l of two floats (about 47 significant bits, relative
// error per operation ~2^-46) on the FP32 and integer pipes. Only the
// position differences stay FP64 instructions (the reference's
// wrappedDifference, src/kernels.cu:1094-1114).
//
// Methods (all from the published literature, written here from the maths):
//   * error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum, and the
//     FMA product error a*b - fl(a*b) (Dekker / Kahan);
//   * double-word sums and products: the "sloppy" sum and the FMA product of
//     Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic
//     building blocks of double-word arithmetic", ACM TOMS 44 (2017);
//   * reciprocal and reciprocal square root: an FP32 estimate, one FP32 Newton
//     step, then one correction from the residual e = 1 - a y (resp. 1 - a y^2)
//     evaluated in double-word: 1/a = y (1 + e + e^2), 1/sqrt(a) = y (1 + e/2 +
//     3 e^2 / 8).
// Conversions between double and float-float are done on the bit patterns
// (integer pipe), so they take no FP64 issue slot.
//
// Functions are __host__ __device__ so the CPU tests evaluate the same code;
// on the host the FP32 estimates come from IEEE division and sqrtf, nudged one
// ulp so the refinement is exercised.
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

#include <cmath>

namespace cbg {

#define CB_HD __host__ __device__ __forceinline__
// Rare slow paths stay calls: inlined, the compiler computes them on every
// call (predicated) and their FP64 instructions take FP64 issue slots.
#ifdef __CUDACC__
#define CB_SLOW static __host__ __device__ __noinline__
#else
#define CB_SLOW static __attribute__((noinline))
#endif

struct ff {
    float h, l;
};

// ---------------------------------------------------------------- bit casts
CB_HD uint32_t ff_fbits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}
CB_HD float ff_bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}
CB_HD uint64_t ff_dbits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return u;
#endif
}
CB_HD double ff_bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    std::memcpy(&d, &u, 8);
    return d;
#endif
}
// The two 32-bit words of a double, and a double from them.
CB_HD uint32_t ff_dhi(double d) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2hiint(d);
#else
    return (uint32_t)(ff_dbits(d) >> 32);
#endif
}
CB_HD uint32_t ff_dlo(double d) {
#ifdef __CUDA_ARCH__
    return (uint32_t)__double2loint(d);
#else
    return (uint32_t)ff_dbits(d);
#endif
}
CB_HD double ff_mkd(uint32_t hi, uint32_t lo) {
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    return ff_bitsd(((uint64_t)hi << 32) | lo);
#endif
}
CB_HD float ff_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
// Plain IEEE operations that the compiler must not contract into an FMA.
CB_HD float ff_mulr(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
CB_HD float ff_addr(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
CB_HD float ff_subr(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

// FP32 estimates (~1 ulp) of 1/a and 1/sqrt(a), a > 0 normal.
CB_HD float ff_rcp_est(float a) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
#else
    return std::nextafterf(1.0f / a, 1e30f);
#endif
}
CB_HD float ff_rsqrt_est(float a) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
#else
    return std::nextafterf(1.0f / std::sqrt(a), 1e30f);
#endif
}

// ------------------------------------------------- error-free transformations
CB_HD ff two_sum(float a, float b) {  // a + b = s + e exactly
    const float s = ff_addr(a, b);
    const float bb = ff_subr(s, a);
    const float e = ff_addr(ff_subr(a, ff_subr(s, bb)), ff_subr(b, bb));
    return {s, e};
}
CB_HD ff fast_two_sum(float a, float b) {  // exact when |a| >= |b| (or a == 0)
    const float s = ff_addr(a, b);
    return {s, ff_subr(b, ff_subr(s, a))};
}

// ------------------------------------------------------ conversions
// The top 24 bits of the significand (truncated) in h; the low 29 bits, rounded
// to their top 23, in l; renormalised so that |l| <= 2^-24 |h|:
// |x - (h + l)| <= 2^-47 |x|. The low part is built without an int -> float
// conversion: the float 1.f 2^(E-23), whose fraction f is those 23 bits, less
// 2^(E-23) (exact). |x| below 2^-103 keeps only the top bits (absolute error
// < 2^-126); below 2^-126 gives 0. |x| must be below 2^128.
CB_HD ff ff_of(double x) {
    // 32-bit words only: 64-bit integer operations cost more issue slots
    const uint32_t hi = ff_dhi(x), lo = ff_dlo(x);
    const uint32_t sign = hi & 0x80000000u;
    const int eb = (int)((hi >> 20) & 0x7ffu);  // biased double exponent
    const int fe = eb - 896;                    // biased float exponent of h
    if (fe <= 0) return {0.0f, 0.0f};
    const uint32_t mant23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const float h = ff_bitsf(sign | ((uint32_t)fe << 23) | mant23);
    const uint32_t rem = lo & 0x1fffffffu;  // the low 29 bits: rem 2^(E-52)
    const int le = fe - 23;                 // biased float exponent of 2^(E-23)
    float l = 0.0f;
    if (le > 0) {
        // (le << 23) + round(rem / 64): a carry out of the fraction gives 2^(E-22)
        const uint32_t one = (uint32_t)le << 23;
        l = ff_subr(ff_bitsf(one + ((rem + 32u) >> 6)), ff_bitsf(one));
    }
    return fast_two_sum(h, sign ? -l : l);
}

// Exact widening of a float (normal or zero) to double on the bit pattern.
CB_HD double ff_f2d(float f) {
    const uint32_t b = ff_fbits(f);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0) return 0.0;
    return ff_mkd((b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3),
                  (b & 7u) << 29);
}

// h + l rounded to double (error <= 1/2 ulp of the double) on the integer
// pipe. Needs |l| <= 2^-24 |h| (a normalised pair: after fast_two_sum), h
// normal or zero. With h's 24-bit significand the sum never reaches the next
// binade; it can fall into the one below only when h is a power of two and l
// has the opposite sign, where the double's ulp is half as large. l in units
// of the double's ulp is below 2^31, so the low word takes it with one carry.
CB_HD double ff_to_double(ff v) {
    const uint32_t hb = ff_fbits(v.h), lb = ff_fbits(v.l);
    const uint32_t he = (hb >> 23) & 0xffu, le = (lb >> 23) & 0xffu;
    if (he == 0) return ff_f2d(v.l);
    const uint32_t dhi = (hb & 0x80000000u) | ((he + 896u) << 20) | ((hb & 0x7fffffu) >> 3);
    const uint32_t dlo = (hb & 7u) << 29;
    if (le == 0) return ff_mkd(dhi, dlo);
    const uint32_t lm = (lb & 0x7fffffu) | 0x800000u;  // 24-bit significand of l
    const bool opp = ((hb ^ lb) & 0x80000000u) != 0;
    const bool down = opp && (hb & 0x7fffffu) == 0;  // h = 2^E, result below 2^E
    // l / ulp(h as double) = lm 2^(le - he + 29); one more bit when down
    const int k = (int)le - (int)he + 29 + (down ? 1 : 0);
    uint32_t delta;
    if (k >= 0) {
        delta = lm << k;  // k <= 6
    } else if (k > -26) {
        delta = (lm + (1u << (-k - 1))) >> (-k);
    } else {
        delta = 0u;
    }
    if (opp) {
        const uint32_t lo2 = dlo - delta;
        return ff_mkd(dhi - (dlo < delta ? 1u : 0u), lo2);
    }
    const uint32_t lo2 = dlo + delta;
    return ff_mkd(dhi + (lo2 < dlo ? 1u : 0u), lo2);
}

// ------------------------------------------------------ arithmetic
CB_HD ff ff_neg(ff a) { return {-a.h, -a.l}; }
CB_HD ff ff_abs(ff a) { return a.h < 0.0f ? ff_neg(a) : a; }
CB_HD ff ff_scale(ff a, float p2) { return {a.h * p2, a.l * p2}; }  // p2 a power of two

// Sloppy double-word sum: relative error ~2^-46 without cancellation; with
// cancellation the absolute error stays ~2^-47 (|a| + |b|).
CB_HD ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.h, b.h);
    const float e = ff_addr(s.l, ff_addr(a.l, b.l));
    return fast_two_sum(s.h, e);
}
CB_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

CB_HD ff ff_mul(ff a, ff b) {
    const float p = ff_mulr(a.h, b.h);
    float e = ff_fma(a.h, b.h, -p);
    e = ff_fma(a.h, b.l, e);
    e = ff_fma(a.l, b.h, e);
    return fast_two_sum(p, e);
}
CB_HD ff ff_mul_f(ff a, float b) {
    const float p = ff_mulr(a.h, b);
    float e = ff_fma(a.h, b, -p);
    e = ff_fma(a.l, b, e);
    return fast_two_sum(p, e);
}
CB_HD ff ff_sqr(ff a) {
    const float p = ff_mulr(a.h, a.h);
    float e = ff_fma(a.h, a.h, -p);
    e = ff_fma(ff_addr(a.h, a.h), a.l, e);
    return fast_two_sum(p, e);
}

// 1/a, a > 0 with a.h a normal float.
CB_HD ff ff_rcp(ff a) {
    float y = ff_rcp_est(a.h);
    y = ff_fma(y, ff_fma(-a.h, y, 1.0f), y);  // FP32 Newton step, |1 - a y| ~ 2^-24
    const float th = ff_mulr(a.h, y);
    float te = ff_fma(a.h, y, -th);
    te = ff_fma(a.l, y, te);
    const float e = ff_subr(ff_subr(1.0f, th), te);  // 1 - a y; 1 - th is exact
    const float c = ff_fma(y, e, ff_mulr(ff_mulr(y, e), e));
    return fast_two_sum(y, c);
}

// 1/sqrt(a), a > 0 with a.h a normal float.
CB_HD ff ff_rsqrt(ff a) {
    float y = ff_rsqrt_est(a.h);
    const float hy = ff_mulr(0.5f, y);
    y = ff_fma(hy, ff_fma(-ff_mulr(a.h, y), y, 1.0f), y);  // FP32 Newton step
    const float sh = ff_mulr(y, y);
    const float sl = ff_fma(y, y, -sh);  // y^2 = sh + sl exactly
    const float th = ff_mulr(a.h, sh);
    float te = ff_fma(a.h, sh, -th);
    te = ff_fma(a.h, sl, te);
    te = ff_fma(a.l, sh, te);
    const float e = ff_subr(ff_subr(1.0f, th), te);  // 1 - a y^2
    const float c = ff_fma(ff_mulr(0.5f, y), e, ff_mulr(ff_mulr(0.375f, e), ff_mulr(e, y)));
    return fast_two_sum(y, c);
}

// sqrt(a) = a / sqrt(a) for a > 0, 0 otherwise.
CB_HD ff ff_sqrt(ff a) {
    if (!(a.h > 0.0f)) return {0.0f, 0.0f};
    return ff_mul(a, ff_rsqrt(a));
}

// a - b evaluated to ~2^-46 (|a| + |b|), as one float: for sign tests.
CB_HD float ff_diff_f(ff a, ff b) {
    const ff s = two_sum(a.h, -b.h);
    return ff_addr(s.h, ff_addr(s.l, ff_subr(a.l, b.l)));
}

// ------------------------------------------- FP64 results with few FP64 ops
// For kernels bound by FP64 issue: full-precision FP64 results whose costly
// parts run on the FP32 and integer pipes.

// A double rounded toward zero to float (normal range), on the bit pattern.
CB_HD float ff_f32(double x) {
    const uint32_t hi = ff_dhi(x), lo = ff_dlo(x);
    const int fe = (int)((hi >> 20) & 0x7ffu) - 896;
    if (fe <= 0) return 0.0f;
    return ff_bitsf((hi & 0x80000000u) | ((uint32_t)fe << 23) | ((hi & 0xfffffu) << 3) |
                    (lo >> 29));
}

// y + c for a double y > 0 and a float c with |c| <= 2^-31 y: c in units of
// the last place of y (below 2^22), rounded to an integer with the 1.5 * 2^23
// shifter and added to y's bit pattern (error <= 1/2 ulp + 2^-7 ulp). The
// FP64 sum when y's exponent is outside [-74, 178], c is larger, or the sum
// leaves y's binade.
CB_SLOW double ff_add_slow(double y, float c) { return y + (double)c; }
CB_HD double ff_add_small(double y, float c) {
    const uint32_t hi = ff_dhi(y), lo = ff_dlo(y);
    const int se = 52 - ((int)((hi >> 20) & 0x7ffu) - 1023) + 127;  // 2^(52 - E)
    const float u = ff_mulr(c, ff_bitsf((uint32_t)(se < 1 ? 1 : se > 254 ? 254 : se) << 23));
    const int d = (int)(ff_fbits(ff_addr(u, 12582912.0f)) - 0x4b400000u);
    const uint32_t lo2 = lo + (uint32_t)d;
    const uint32_t hi2 = hi + (d < 0 ? 0xffffffffu : 0u) + (lo2 < lo ? 1u : 0u);
    if (se < 1 || se > 254 || !(fabsf(u) < 4194304.0f) || ((hi2 ^ hi) & 0x7ff00000u))
        return ff_add_slow(y, c);
    return ff_mkd(hi2, lo2);
}

// Leading zeros of a 32-bit word (32 for 0).
CB_HD int ff_clz(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __clz((int)x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

// a - b, equal to the IEEE FP64 subtraction bit for bit, on the integer pipe
// when it needs no rounding and the operands are alike: same sign, normal,
// biased exponents above 64 and at most one apart, and |a| - |b| within 53
// significant bits (Sterbenz's case b/2 <= a <= 2b always is: two nearby
// positions, a position and its update). Then the difference of the integer
// significands (the larger exponent's shifted left by one) is exact, and is
// renormalised with a count of leading zeros. Everything else: the FP64
// subtraction, as a call.
CB_SLOW double sub_slow(double a, double b) { return a - b; }
CB_HD double sub_exact(double a, double b) {
    const uint32_t ah = ff_dhi(a), al = ff_dlo(a), bh = ff_dhi(b), bl = ff_dlo(b);
    const int ea = (int)((ah >> 20) & 0x7ffu), eb = (int)((bh >> 20) & 0x7ffu);
    const int d = ea - eb;
    // significands with the hidden bit as (high, low) words
    uint32_t mah = (ah & 0xfffffu) | 0x100000u, mal = al;
    uint32_t mbh = (bh & 0xfffffu) | 0x100000u, mbl = bl;
    if (d > 0) {
        mah = (mah << 1) | (mal >> 31);
        mal <<= 1;
    } else if (d < 0) {
        mbh = (mbh << 1) | (mbl >> 31);
        mbl <<= 1;
    }
    // D = Ma - Mb over 64 bits, then |D|
    uint32_t dl = mal - mbl;
    uint32_t dh = mah - mbh - (mal < mbl ? 1u : 0u);
    const bool neg = (dh & 0x80000000u) != 0;
    if (neg) {
        dl = 0u - dl;
        dh = ~dh + (dl == 0u ? 1u : 0u);
    }
    const bool ok = ((ah ^ bh) & 0x80000000u) == 0u && ea > 64 && eb > 64 && ea < 0x7ff &&
                    eb < 0x7ff && d >= -1 && d <= 1 && dh < 0x200000u;  // |D| < 2^53
    if (!ok) return sub_slow(a, b);
    if ((dh | dl) == 0u) return 0.0;  // +0, as IEEE round-to-nearest
    const int lz = dh ? ff_clz(dh) : 32 + ff_clz(dl);  // 11 .. 63
    const int sh = lz - 11;                            // leading bit to bit 52
    uint32_t mh, ml;
    if (sh >= 32) {
        mh = dl << (sh - 32);
        ml = 0u;
    } else if (sh > 0) {
        mh = (dh << sh) | (dl >> (32 - sh));
        ml = dl << sh;
    } else {
        mh = dh;
        ml = dl;
    }
    const uint32_t e = (uint32_t)((ea < eb ? ea : eb) - sh);  // > 11
    const uint32_t sign = (ah & 0x80000000u) ^ (neg ? 0x80000000u : 0u);
    return ff_mkd(sign | (e << 20) | (mh & 0xfffffu), ml);
}

// true when a > 0 and float-float holds a, its root and reciprocal root
CB_HD bool ff_in_range(double a) {
    const int eb = (int)((ff_dhi(a) >> 20) & 0xfffu);  // sign bit included: a > 0 only
    return eb > 1023 - 100 && eb < 1023 + 100;
}

// 1/sqrt(a) to ~1 ulp with 2 FP64 instructions, for ff_in_range(a): a
// float-float estimate (~2^-46) widened to double, the residual
// e = 1 - a y^2 in FP64, and the correction y e / 2 (~2^-46 y, needed to 8
// bits) in FP32, added on the integer pipe.
CB_HD double rsqrt_d_core(double a) {
    const double y = ff_to_double(ff_rsqrt(ff_of(a)));
    const double t = a * y;
    const double e = fma(-t, y, 1.0);
    return ff_add_small(y, ff_mulr(ff_mulr(0.5f, ff_f32(y)), ff_f32(e)));
}

// 1/a to ~1 ulp with 1 FP64 instruction (as rsqrt_d_core, e = 1 - a y).
CB_HD double rcp_d_core(double a) {
    const double y = ff_to_double(ff_rcp(ff_of(a)));
    const double e = fma(-a, y, 1.0);
    return ff_add_small(y, ff_mulr(ff_f32(y), ff_f32(e)));
}

// sqrt(a) in float-float (~2^-46 relative) rounded to double, no FP64
// instruction; 0 for a <= 0; IEEE sqrt outside the float-float range.
CB_SLOW double sqrt_slow(double a) { return a > 0.0 ? sqrt(a) : 0.0; }
CB_HD double sqrt_ffd(double a) {
    if (!ff_in_range(a)) return sqrt_slow(a);  // also a <= 0
    return ff_to_double(ff_sqrt(ff_of(a)));
}

#undef CB_HD
#undef CB_SLOW

}  // namespace cbg
