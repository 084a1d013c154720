/* Exact stencil sums for the device Laplacian.
 *
 * On GB300 an FP64 add or fused multiply-add issues at about 1.9 lanes per
 * clock per SM, while 32-bit integer instructions issue at full rate.  The
 * ring sums of a Laplacian are therefore accumulated here in 64-bit
 * integers instead of FP64: every stencil value x = +-M 2^(e-1075) (M the
 * 53-bit significand, e the biased exponent, e >= 1) is written as the
 * integer +-round(M / 2^(A+G-e)) in units of 2^(A+G-1075), where A is the
 * largest exponent among the values of this one stencil and G guard bits
 * keep the weighted sum below 2^63.  Integer adds and the small integer
 * weights of the stencil are exact; the only roundings are the shifted-out
 * significand bits of values smaller than the largest one (each at most
 * 2^(A+G-1076), half a unit in the last place of the largest value for
 * G = 0) and one final conversion of the 64-bit sum to FP64.  The FP64
 * evaluation rounds after every add instead; on stencils with strong
 * cancellation the integer sum's error is below the FP64 sum's for the 7-
 * and 13-point Laplacians and comparable for the 19-point one (two guard
 * bits).  The result scales exactly with powers of two of the input and is
 * independent of the cell's position.
 *
 * A stencil whose largest value is not finite falls back to FP64 so that
 * NaN and infinity propagate as they do in the reference; values below
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

/* Biased exponent, at least 1 (subnormals share the exponent of 2^-1022). */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE int expo(long long b) {
    const int e = (int)((b >> 52) & 0x7FF);
    return e > 0 ? e : 1;
}

/* +-round(M / 2^shift) (halves away from zero) for the value with bit
 * pattern b; shift in [0, 63]. */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE long long term(long long b, int shift) {
    const unsigned long long frac = (unsigned long long)b & 0xFFFFFFFFFFFFFull;
    const unsigned long long M = frac | ((b & 0x7FF0000000000000ll) ? (1ull << 52) : 0ull);
    const unsigned long long m = (M + ((1ull << shift) >> 1)) >> shift;
    return b < 0 ? -(long long)m : (long long)m;
}

/* Smallest anchor exponent: values below 2^(kMinAnchor - 1075) vanish. */
constexpr int kMinAnchor = 128;

/* Exact weighted sum  sum_r w[r] * (sum of the values of ring r)  times
 * `scale` (a positive FP64 factor applied after the single rounding of the
 * integer sum).  Ring r has n[r] values; v lists the rings one after the
 * other.  G guard bits must satisfy 2^53 * sum_r |w[r]| n[r] < 2^(63+G). */
template <int NV, int NR, int G>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
weighted_sum(const double (&v)[NV], const int (&n)[NR], const long long (&w)[NR],
             double scale) {
    long long b[NV];
    int A = kMinAnchor;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        b[q] = bits(v[q]);
        const int e = expo(b[q]);
        A = e > A ? e : A;
    }
    if (A == 0x7FF) {
        /* NaN or infinity: FP64 sums in ring order */
        double acc = 0.;
        int q = 0;
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            double s = 0.;
            for (int t = 0; t < n[r]; ++t) s += v[q++];
            acc += (double)w[r] * s;
        }
        return acc * scale;
    }
    const int top = A + G;
    long long acc = 0;
    int q = 0;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        long long s = 0;
#pragma unroll
        for (int t = 0; t < n[r]; ++t, ++q) {
            const int sh = top - expo(b[q]);
            s += term(b[q], sh < 63 ? sh : 63);
        }
        acc += w[r] * s;
    }
    /* acc * 2^(top - 1075) * scale, rounded once by the conversion and once
     * by the product with scale; the power of two goes straight into the
     * exponent field when the result is a normal number */
    const double r = (double)acc * scale;
    if (r == 0.) return r;
    const long long rb = bits(r);
    const int er = (int)((rb >> 52) & 0x7FF) + (top - 1075);
    if (er >= 1 && er <= 2046) return from_bits(rb + ((long long)(top - 1075) << 52));
    return scalbn(r, top - 1075);
}

} // namespace fixed
} // namespace utils
} // namespace sledgehamr

#endif // SH_FIXED_STENCIL_H_
