/* Finite-difference stencils of the sledgehamr plugin surface:
 * sledgehamr::utils::Laplacian<order> and sledgehamr::utils::Gradient<order>
 * for order 0..3, plus the constexpr_for helper that project code uses.
 *
 * Reference: source/utils/sledgehamr_utils.h:11-17 (constexpr_for),
 *            :50-94 (Laplacian<0..3>), :106-188 (Gradient<0..3>).
 *
 * The coefficients are those of the standard central difference formulas:
 *   order 1 (2nd-order accurate, 7 points):  (S1 - 6 c) / dx^2
 *   order 2 (4th-order, 13 points):  (-S2 + 16 S1 - 90 c) / (12 dx^2)
 *   order 3 (6th-order, 19 points):  (2 S3 - 27 S2 + 270 S1 - 1470 c) / (180 dx^2)
 * where Sr is the sum of the six neighbours at distance r along the axes,
 * accumulated in the order +x, -x, +y, -y, +z, -z.  The division by the
 * denominator is done as a multiplication by its reciprocal: that
 * reciprocal is loop invariant and is hoisted out of cell loops, which
 * matters on GB300 where an FP64 division costs about as much as ten FP64
 * fused multiply-adds.  The result differs from a true division by at most
 * one rounding.
 *
 * Device code (unless SH_STENCIL_FP64 is defined) evaluates the Laplacians
 * and the Gradients of orders 2 and 3 with their weighted sums accumulated
 * exactly in 64-bit integers (sh_fixed_stencil.h) instead of FP64 adds: the
 * same formulas, one rounding of the sum instead of one per add, and far
 * fewer FP64 instructions, which GB300 issues at 1/64 of its FP32 rate.
 * Host code keeps the FP64 evaluation order above.
 */
#ifndef SLEDGEHAMR_SLEDGEHAMR_UTILS_H_
#define SLEDGEHAMR_SLEDGEHAMR_UTILS_H_

#include <type_traits>
#include <utility>

#include "sh_amrex.h"
#include "sh_fixed_stencil.h"

namespace sledgehamr {
namespace utils {

/* Compile-time loop: calls f(std::integral_constant<..., i>) for
 * i = Start, Start+Inc, ... < End. */
template <auto Start, auto End, auto Inc, class F>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr void constexpr_for(F &&f) {
    if constexpr (Start < End) {
        f(std::integral_constant<decltype(Start), Start>());
        constexpr_for<Start + Inc, End, Inc>(f);
    }
}

namespace detail {

/* Sum of the six axis neighbours of (i,j,k) at distance r. */
template <class A4>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
axis_ring_sum(const A4 &s, int i, int j, int k, int c, int r) {
    double acc = s(i + r, j, k, c);
    acc += s(i - r, j, k, c);
    acc += s(i, j + r, k, c);
    acc += s(i, j - r, k, c);
    acc += s(i, j, k + r, c);
    acc += s(i, j, k - r, c);
    return acc;
}

/* Weights of the Laplacian rings: r = 0 is the centre cell. */
template <int Order>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr double lap_ring(int r) {
    if constexpr (Order == 1) {
        return r == 0 ? -6. : 1.;
    } else if constexpr (Order == 2) {
        return r == 0 ? -90. : (r == 1 ? 16. : -1.);
    } else {
        return r == 0 ? -1470. : (r == 1 ? 270. : (r == 2 ? -27. : 2.));
    }
}
template <int Order>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr double lap_denom() {
    return Order == 1 ? 1. : (Order == 2 ? 12. : 180.);
}

/* Offset of cell (i,j,k) by d along axis 'x', 'y' or 'z'. */
template <class A4>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
along(const A4 &s, int i, int j, int k, int c, char axis, int d) {
    return axis == 'x' ? s(i + d, j, k, c)
                       : (axis == 'y' ? s(i, j + d, k, c) : s(i, j, k + d, c));
}

/* The Laplacian with its ring sums accumulated exactly in 64-bit integers
 * (sh_fixed_stencil.h): centre, then the rings r = 1..Order with the integer
 * weights of lap_ring, one rounding of the sum, then the product with
 * 1 / (denominator dx^2). */
template <int Order, class A4>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
laplacian_fixed(const A4 &s, int i, int j, int k, int c, double dx2) {
    constexpr int NV = 6 * Order + 1;
    double v[NV];
    int n[Order + 1];
    long long w[Order + 1];
    v[0] = s(i, j, k, c);
    n[0] = 1;
    w[0] = (long long)lap_ring<Order>(0);
#pragma unroll
    for (int r = 1; r <= Order; ++r) {
        v[6 * r - 5] = s(i + r, j, k, c);
        v[6 * r - 4] = s(i - r, j, k, c);
        v[6 * r - 3] = s(i, j + r, k, c);
        v[6 * r - 2] = s(i, j - r, k, c);
        v[6 * r - 1] = s(i, j, k + r, c);
        v[6 * r] = s(i, j, k - r, c);
        n[r] = 6;
        w[r] = (long long)lap_ring<Order>(r);
    }
    /* 2^53 * sum |w| n = 2^53 * {12, 192, 3264}: headroom of 6 and 2 bits
     * below 2^63 for orders 1 and 2, two bits short for order 3 */
    return fixed::weighted_sum<NV, Order + 1, Order == 1 ? -6 : (Order == 2 ? -2 : 2)>(
        v, n, w, 1. / (lap_denom<Order>() * dx2));
}

/* Gradient<2> and <3> the same way: the 4 or 6 values along the axis with
 * the integer weights of the central difference, one rounding of the sum,
 * then the product with 1 / (denominator dx). */
template <int Order, class A4>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
gradient_fixed(const A4 &s, int i, int j, int k, int c, double dx, char axis) {
    static_assert(Order == 2 || Order == 3, "orders 2 and 3");
    constexpr int NV = 2 * Order;
    double v[NV];
    int n[NV];
    long long w[NV];
    if constexpr (Order == 2) {
        /* -f(+2) + 8 f(+1) + f(-2) - 8 f(-1) */
        constexpr int off[4] = {2, 1, -2, -1};
        constexpr long long wt[4] = {-1, 8, 1, -8};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[q] = along(s, i, j, k, c, axis, off[q]);
            n[q] = 1;
            w[q] = wt[q];
        }
        /* 2^53 * sum |w| = 2^53 * 18: five bits of headroom */
        return fixed::weighted_sum<NV, NV, -5>(v, n, w, 1. / (12. * dx));
    } else {
        /* f(+3) - f(-3) - 9 f(+2) + 9 f(-2) + 45 f(+1) - 45 f(-1) */
        constexpr int off[6] = {3, -3, 2, -2, 1, -1};
        constexpr long long wt[6] = {1, -1, -9, 9, 45, -45};
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            v[q] = along(s, i, j, k, c, axis, off[q]);
            n[q] = 1;
            w[q] = wt[q];
        }
        /* 2^53 * sum |w| = 2^53 * 110: three bits of headroom */
        return fixed::weighted_sum<NV, NV, -3>(v, n, w, 1. / (60. * dx));
    }
}

} // namespace detail

template <int Order>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
Laplacian(amrex::Array4<amrex::Real const> const &state, const int i,
          const int j, const int k, const int c, const double dx2) {
    if constexpr (Order == 0) {
        return 0.;
    } else {
#if defined(__CUDA_ARCH__) && !defined(SH_STENCIL_FP64)
        return detail::laplacian_fixed<Order>(state, i, j, k, c, dx2);
#else
        /* outermost ring first, centre last */
        double acc = detail::lap_ring<Order>(Order) *
                     detail::axis_ring_sum(state, i, j, k, c, Order);
        constexpr_for<1, Order, 1>([&](auto q) {
            constexpr int r = Order - q;
            acc += detail::lap_ring<Order>(r) *
                   detail::axis_ring_sum(state, i, j, k, c, r);
        });
        acc += detail::lap_ring<Order>(0) * state(i, j, k, c);
        return acc * (1. / (detail::lap_denom<Order>() * dx2));
#endif
    }
}

template <int Order>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
Gradient(amrex::Array4<amrex::Real const> const &state, const int i,
         const int j, const int k, const int c, const double dx,
         const char axis) {
    using detail::along;
#if defined(__CUDA_ARCH__) && !defined(SH_STENCIL_FP64)
    if constexpr (Order >= 2) {
        return detail::gradient_fixed<Order>(state, i, j, k, c, dx, axis);
    } else
#endif
    if constexpr (Order == 0) {
        return 0.;
    } else if constexpr (Order == 1) {
        /* (f(+1) - f(-1)) / (2 dx) */
        return (along(state, i, j, k, c, axis, 1) -
                along(state, i, j, k, c, axis, -1)) *
               (1. / (2. * dx));
    } else if constexpr (Order == 2) {
        /* (-f(+2) + 8 f(+1) + f(-2) - 8 f(-1)) / (12 dx) */
        double acc = -along(state, i, j, k, c, axis, 2);
        acc += 8. * along(state, i, j, k, c, axis, 1);
        acc += along(state, i, j, k, c, axis, -2);
        acc -= 8. * along(state, i, j, k, c, axis, -1);
        return acc * (1. / (12. * dx));
    } else {
        /* (f(+3) - f(-3) - 9 f(+2) + 9 f(-2) + 45 f(+1) - 45 f(-1)) / (60 dx) */
        double acc = along(state, i, j, k, c, axis, 3);
        acc -= along(state, i, j, k, c, axis, -3);
        acc -= 9. * along(state, i, j, k, c, axis, 2);
        acc += 9. * along(state, i, j, k, c, axis, -2);
        acc += 45. * along(state, i, j, k, c, axis, 1);
        acc -= 45. * along(state, i, j, k, c, axis, -1);
        return acc * (1. / (60. * dx));
    }
}

} // namespace utils
} // namespace sledgehamr

#endif // SLEDGEHAMR_SLEDGEHAMR_UTILS_H_
