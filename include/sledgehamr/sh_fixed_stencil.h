/* Exact stencil sums for the device Laplacian.
 *
 * On GB300 an FP64 add or fused multiply-add issues at about 1.9 lanes per
 * clock per SM, while 32-bit integer instructions issue at full rate.  The
 * ring sums of a Laplacian are therefore accumulated here in 64-bit
 * integers instead of FP64: every stencil value x = +-M 2^(e-1075) (M the
 * 53-bit significand, e the biased exponent, e >= 1) is written as the
 * integer +-M 2^(e-A-G) in units of 2^(A+G-1075), where A is the largest
 * exponent among the values of this one stencil and G is chosen per stencil
 * so that the weighted sum stays below 2^63 (G = -6 for the 7-point, -2 for
 * the 13-point and +2 for the 19-point Laplacian).  Integer adds and the
 * small integer weights of the stencil are exact; the only roundings are
 * the significand bits shifted out of values smaller than the largest one
 * (each below 2^G units in the last place of the largest value) and one
 * final conversion of the 64-bit sum to FP64.  The FP64 evaluation rounds
 * after every add instead; on stencils with strong cancellation the integer
 * sum's error is below the FP64 sum's for the 7- and 13-point Laplacians
 * and comparable for the 19-point one.  The result scales exactly with
 * powers of two of the input and is independent of the cell's position.
 *
 * A stencil holding NaN or infinity gives NaN (the FP64 evaluation gives
 * NaN or an infinity there: either way the run has diverged); values below
 * 2^-947 are treated as zero.
 */
#ifndef SH_FIXED_STENCIL_H_
#define SH_FIXED_STENCIL_H_

#include <cmath>
#include <cstring>

#include "sh_amrex.h"

namespace sledgehamr {
namespace utils {
namespace fixed {

AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE long long bits(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    long long b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double from_bits(long long b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

/* High and low 32-bit words of a double. */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int hi_word(double x) {
#if defined(__CUDA_ARCH__)
    return __double2hiint(x);
#else
    return (int)(bits(x) >> 32);
#endif
}
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE unsigned lo_word(double x) {
#if defined(__CUDA_ARCH__)
    return (unsigned)__double2loint(x);
#else
    return (unsigned)bits(x);
#endif
}

/* Biased exponent from the high word (0 for zeros and subnormals). */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int expo(int hi) { return (hi >> 20) & 0x7FF; }

/* Significand with the implicit bit, times 2^P.  The implicit bit is set for
 * zeros and subnormals too: their exponent is at least kMinAnchor below the
 * anchor, so the shift below removes them entirely. */
template <int P>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE unsigned long long significand(int hi, unsigned lo) {
    const unsigned long long m =
        ((unsigned long long)(((unsigned)hi & 0xFFFFFu) | 0x100000u) << 32) | lo;
    return m << P;
}

/* Smallest anchor exponent: values below 2^(kMinAnchor - 1075) vanish. */
constexpr int kMinAnchor = 128;

/* acc * 2^pw * scale: one rounding in the conversion of acc, one in the
 * product with scale (a positive factor); the power of two goes straight
 * into the exponent field when the result is a normal number. */
#if defined(__CUDA_ARCH__)
/* The rare paths live in functions of their own so that the compiler keeps
 * them behind a branch instead of predicating their FP64 instructions into
 * every call. */
__device__ __noinline__ double scale_pow2_slow(double res, int pw) { return scalbn(res, pw); }
#else
inline double scale_pow2_slow(double res, int pw) { return std::scalbn(res, pw); }
#endif

AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int clz64(unsigned long long u) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)u);
#else
    return __builtin_clzll(u);
#endif
}

/* Bits of the FP64 value nearest to acc * 2^pw (ties to even), for acc != 0
 * with |acc| < 2^63, formed with integer instructions only; the biased
 * exponent goes to *e (the bits are valid when 1 <= *e <= 2046).  On
 * GB300 the integer-to-FP64 conversion instruction issues on the narrow
 * FP64 pipe; these integer steps issue on the integer pipe. */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE unsigned long long int_to_f64_bits(long long acc, int pw,
                                                                            int *e) {
    const unsigned long long sign = acc < 0 ? (1ull << 63) : 0ull;
    const unsigned long long u = acc < 0 ? 0ull - (unsigned long long)acc : (unsigned long long)acc;
    const int lz = clz64(u);
    const unsigned long long nrm = u << lz; /* leading one at bit 63 */
    unsigned long long mant = nrm >> 11;    /* 53 bits with the leading one */
    const unsigned rem = (unsigned)(nrm & 0x7FFull);
    mant += (unsigned long long)((rem > 0x400u) | ((rem == 0x400u) & (unsigned)(mant & 1ull)));
    const int carry = (int)(mant >> 53); /* rounded up to 2^53 */
    mant >>= carry;
    *e = 63 - lz + 1023 + pw + carry;
    return sign | ((unsigned long long)(unsigned)*e << 52) | (mant & 0xFFFFFFFFFFFFFull);
}

/* log2 of x when x is a positive normal power of two, else -2000. */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int pow2_exponent(double x) {
    const long long b = bits(x);
    const int ex = (int)((b >> 52) & 0x7FF);
    return (b > 0 && (b & 0xFFFFFFFFFFFFFll) == 0 && ex >= 1 && ex <= 2046) ? ex - 1023 : -2000;
}

AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double to_double(long long acc, int pw) {
    if (acc == 0) return 0.;
    int e;
    const unsigned long long rb = int_to_f64_bits(acc, pw, &e);
    if (e >= 1 && e <= 2046) return from_bits((long long)rb);
    return scale_pow2_slow((double)acc, pw);
}
/* acc * 2^pw * scale: a power-of-two scale (1 / dx^2 for dx a power of two)
 * joins the exponent, so the result takes one rounding and no FP64
 * instruction; any other scale costs one FP64 product after the rounded
 * conversion. */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double to_double(long long acc, int pw, double scale) {
    if (acc == 0) return 0.;
    const int ps = pow2_exponent(scale);
    const bool p2 = ps != -2000;
    int e;
    /* one conversion for both cases: with the power of two folded in, or
     * of acc alone (|acc| < 2^63 converts to a normal number) */
    const unsigned long long cb = int_to_f64_bits(acc, p2 ? pw + ps : 0, &e);
    if (p2) {
        if (e >= 1 && e <= 2046) return from_bits((long long)cb);
        return scale_pow2_slow((double)acc, pw + ps);
    }
    const double res = from_bits((long long)cb) * scale;
    const long long rb = bits(res);
    const int er = (int)((rb >> 52) & 0x7FF) + pw;
    if (er >= 1 && er <= 2046) return from_bits(rb + ((long long)pw << 52));
    return scale_pow2_slow(res, pw);
}

/* +-M 2^(e-A+P) truncated toward zero: the value with high word hi and low
 * word lo in units of 2^(A-P-1075), for an anchor A >= its exponent. */
template <int P>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE long long to_fixed(int hi, unsigned lo, int A) {
    const int d = A - expo(hi);
    const unsigned long long m = significand<P>(hi, lo) >> (d < 63 ? d : 63);
    return hi < 0 ? -(long long)m : (long long)m;
}

/* Largest exponent of n values (at least kMinAnchor); hi receives their
 * high words. */
template <int NV>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int anchor(const double (&v)[NV], int (&hi)[NV]) {
    int A = kMinAnchor;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        hi[q] = hi_word(v[q]);
        const int e = expo(hi[q]);
        A = e > A ? e : A;
    }
    return A;
}

/* Exact weighted sum  sum_r w[r] * (sum of the values of ring r)  times
 * `scale` (a positive FP64 factor applied after the single rounding of the
 * integer sum).  Ring r has n[r] values; v lists the rings one after the
 * other.  The unit of the integer sum is 2^(A+G-1075) with A the largest
 * exponent of the stencil:
 *   G <= 0: every significand is shifted left by -G (the headroom that the
 *           stencil's weights leave below 2^63) and then right by A - e with
 *           truncation, so each term is low by less than 2^G units in the
 *           last place of the largest value;
 *   G > 0:  significands are shifted right by A + G - e with rounding to
 *           nearest (at most half a unit of 2^G ulps).
 * G must satisfy 2^(53-G) * sum_r |w[r]| n[r] < 2^63.  Positive and negative
 * terms go to separate accumulators, so no term is negated. */
template <int NV, int NR, int G>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
weighted_sum(const double (&v)[NV], const int (&n)[NR], const long long (&w)[NR],
             double scale) {
    int hi[NV];
    const int A = anchor(v, hi);
    if (A == 0x7FF) return from_bits(0x7FF8000000000000ll); /* NaN or infinity: NaN */
    constexpr int P = G < 0 ? -G : 0;
    constexpr int R = G > 0 ? G : 0;
    long long acc = 0;
    int q = 0;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        unsigned long long sp = 0, sn = 0;
#pragma unroll
        for (int t = 0; t < n[r]; ++t, ++q) {
            const int d = A + R - expo(hi[q]);
            const int sh = d < 63 ? d : 63;
            const unsigned long long M = significand<P>(hi[q], lo_word(v[q]));
            const unsigned long long m =
                R > 0 ? (M + ((1ull << sh) >> 1)) >> sh : M >> sh;
            if (hi[q] < 0)
                sn += m;
            else
                sp += m;
        }
        acc += w[r] * (long long)(sp - sn);
    }
    /* acc * 2^(A + G - 1075) * scale, rounded once by the conversion and once
     * by the product with scale */
    return to_double(acc, A + G - 1075, scale);
}

} // namespace fixed
} // namespace utils
} // namespace sledgehamr

#endif // SH_FIXED_STENCIL_H_
