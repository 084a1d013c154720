/* Host check of the integer-accumulated Laplacian of
 * include/sledgehamr/sh_fixed_stencil.h against the exact value (binary128)
 * and against the FP64 evaluation of the reference's formula, on stencils
 * with strong cancellation (smooth fields), mixed magnitudes, zeros,
 * subnormal-range values, NaN and infinity.  Prints one line per order:
 *   order max_err_fixed max_err_fp64   (units: ulp of the largest term / (denom dx^2))
 * and exits non-zero when a property fails (error above the FP64 error for
 * the 7- and 13-point stencils, above 1.25 times it for the 19-point one;
 * inexact scaling by -4; wrong zeros, NaN or infinity). */
#include <cmath>
#include <cstdio>
#include <random>

#include <quadmath.h>
#include <sledgehamr_utils.h>

using namespace sledgehamr::utils;

namespace {

constexpr int N = 7, C0 = (3 * N + 3) * N + 3;

template <int Order>
double fixed_lap(const double *a, double dx2) {
    amrex::Array4<const double> s(a, N, N * N, N * N * N, amrex::Dim3{0, 0, 0},
                                  amrex::Dim3{N, N, N}, 1);
    return detail::laplacian_fixed<Order>(s, 3, 3, 3, 0, dx2);
}
template <int Order>
double fp64_lap(const double *a, double dx2) {
    amrex::Array4<const double> s(a, N, N * N, N * N * N, amrex::Dim3{0, 0, 0},
                                  amrex::Dim3{N, N, N}, 1);
    return Laplacian<Order>(s, 3, 3, 3, 0, dx2);
}
template <int Order>
double exact_lap(const double *a, double dx2) {
    __float128 acc = (__float128)detail::lap_ring<Order>(0) * a[C0];
    for (int r = 1; r <= Order; ++r) {
        const int offs[6] = {r, -r, r * N, -r * N, r * N * N, -r * N * N};
        for (int o : offs) acc += (__float128)detail::lap_ring<Order>(r) * a[C0 + o];
    }
    return (double)(acc / ((__float128)detail::lap_denom<Order>() * dx2));
}

template <int Order>
bool run(std::mt19937_64 &g) {
    std::normal_distribution<double> nd;
    double ef = 0, e64 = 0;
    const double dx2 = 0.0625 * 0.0625;
    double a[N * N * N], b[N * N * N];
    for (int it = 0; it < 100000; ++it) {
        const double base = nd(g) * std::pow(10., (int)(g() % 40) - 20);
        for (int q = 0; q < N * N * N; ++q)
            a[q] = base * (1 + 1e-3 * nd(g)) + (it % 7 == 0 ? base * nd(g) : 0.);
        if (it % 11 == 0) a[C0] = 0.;
        if (it % 13 == 0) a[C0 + 1] = -a[C0 + 1] * 1e-30;
        double mx = 0;
        for (int q = 0; q < N * N * N; ++q) mx = std::fmax(mx, std::fabs(a[q]));
        const double unit = std::ldexp(1.0, std::ilogb(mx) - 52) /
                            (detail::lap_denom<Order>() * dx2);
        const double ex = exact_lap<Order>(a, dx2);
        const double f = fixed_lap<Order>(a, dx2);
        ef = std::fmax(ef, std::fabs(f - ex) / unit);
        e64 = std::fmax(e64, std::fabs(fp64_lap<Order>(a, dx2) - ex) / unit);
        /* exact scaling by powers of two, odd symmetry */
        for (int q = 0; q < N * N * N; ++q) b[q] = -4. * a[q];
        if (fixed_lap<Order>(b, dx2) != -4. * f) {
            std::printf("scaling failed, order %d\n", Order);
            return false;
        }
    }
    std::printf("%d %.3f %.3f\n", Order, ef, e64);
    /* orders 1 and 2 (no guard bits) are at least as accurate as FP64; the
     * 19-point stencil drops two guard bits and stays within 25 % of it */
    if (ef > e64 * (Order == 3 ? 1.25 : 1.0001) + 1.0) {
        std::printf("fixed error above the FP64 error, order %d\n", Order);
        return false;
    }
    /* special values */
    for (int q = 0; q < N * N * N; ++q) a[q] = 0.;
    if (fixed_lap<Order>(a, dx2) != 0.) return false;
    a[C0 + N] = 1.0;
    if (fixed_lap<Order>(a, dx2) != fp64_lap<Order>(a, dx2)) return false;
    a[C0] = NAN;
    if (!std::isnan(fixed_lap<Order>(a, dx2))) return false;
    a[C0] = INFINITY;
    if (!std::isnan(fixed_lap<Order>(a, dx2))) return false;
    return true;
}

template <int Order>
bool run_gradient(std::mt19937_64 &g) {
    std::normal_distribution<double> nd;
    double ef = 0, e64 = 0;
    const double dx = 0.0625;
    double a[N * N * N], b[N * N * N];
    amrex::Array4<const double> s(a, N, N * N, N * N * N, amrex::Dim3{0, 0, 0},
                                  amrex::Dim3{N, N, N}, 1);
    amrex::Array4<const double> sb(b, N, N * N, N * N * N, amrex::Dim3{0, 0, 0},
                                   amrex::Dim3{N, N, N}, 1);
    const double w2[4] = {-1, 8, 1, -8};
    const int o2[4] = {2, 1, -2, -1};
    const double w3[6] = {1, -1, -9, 9, 45, -45};
    const int o3[6] = {3, -3, 2, -2, 1, -1};
    for (int it = 0; it < 100000; ++it) {
        const double base = nd(g) * std::pow(10., (int)(g() % 40) - 20);
        for (int q = 0; q < N * N * N; ++q)
            a[q] = base * (1 + 1e-3 * nd(g)) + (it % 7 == 0 ? base * nd(g) : 0.);
        const char axis = "xyz"[it % 3];
        const int stride = axis == 'x' ? 1 : (axis == 'y' ? N : N * N);
        __float128 acc = 0;
        double mx = 0;
        for (int t = 0; t < 2 * Order; ++t) {
            const int o = Order == 2 ? o2[t] : o3[t];
            acc += (__float128)(Order == 2 ? w2[t] : w3[t]) * a[C0 + o * stride];
            mx = std::fmax(mx, std::fabs(a[C0 + o * stride]));
        }
        const double den = Order == 2 ? 12. : 60.;
        const double ex = (double)(acc / ((__float128)den * dx));
        const double unit = std::ldexp(1.0, std::ilogb(mx) - 52) / (den * dx);
        const double f = detail::gradient_fixed<Order>(s, 3, 3, 3, 0, dx, axis);
        ef = std::fmax(ef, std::fabs(f - ex) / unit);
        e64 = std::fmax(e64, std::fabs(Gradient<Order>(s, 3, 3, 3, 0, dx, axis) - ex) / unit);
        for (int q = 0; q < N * N * N; ++q) b[q] = -4. * a[q];
        if (detail::gradient_fixed<Order>(sb, 3, 3, 3, 0, dx, axis) != -4. * f) {
            std::printf("gradient scaling failed, order %d\n", Order);
            return false;
        }
    }
    std::printf("g%d %.3f %.3f\n", Order, ef, e64);
    if (ef > e64 * 1.0001 + 1.0) {
        std::printf("fixed gradient error above the FP64 error, order %d\n", Order);
        return false;
    }
    return true;
}

/* The integer-only conversion equals the FP64 conversion (round to nearest,
 * ties to even) times 2^pw, on random magnitudes, exact ties and carries. */
bool run_conversion(std::mt19937_64 &g) {
    long long checked = 0;
    for (int it = 0; it < 2000000; ++it) {
        const int nb = 1 + (int)(g() % 63);
        unsigned long long u = g() >> (64 - nb);
        if (it % 5 == 1 && nb > 54) { /* exact tie below the 53 kept bits */
            const int k = nb - 53;
            u = ((u | 1ull << (nb - 1)) & ~((1ull << k) - 1)) | (1ull << (k - 1));
        }
        if (it % 5 == 2 && nb > 54) u = (1ull << nb) - 1; /* rounds up into a carry */
        if (u == 0 || u >= (1ull << 63)) continue;
        const long long acc = (g() & 1) ? -(long long)u : (long long)u;
        const int pw = (int)(g() % 1200) - 700;
        const double want = std::ldexp((double)acc, pw);
        if (!std::isnormal(want)) continue;
        const double got = fixed::to_double(acc, pw);
        if (got != want) {
            std::printf("conversion failed: %lld * 2^%d\n", acc, pw);
            return false;
        }
        const double sc = (it % 3 == 0) ? 0.25 : 1.0 / 12.0;
        const double ws = std::ldexp((double)acc * sc, pw);
        if (std::isnormal(ws) && fixed::to_double(acc, pw, sc) != ws) {
            std::printf("scaled conversion failed: %lld * %g * 2^%d\n", acc, sc, pw);
            return false;
        }
        ++checked;
    }
    std::printf("c %lld\n", checked);
    return true;
}

} // namespace

int main() {
    std::mt19937_64 g(12345);
    const bool ok = run_conversion(g) && run<1>(g) && run<2>(g) && run<3>(g) &&
                    run_gradient<2>(g) && run_gradient<3>(g);
    return ok ? 0 : 1;
}
