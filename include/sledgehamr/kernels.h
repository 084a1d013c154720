/* Per-cell kernels of the sledgehamr core that project code and the level
 * synchroniser call: the 2x2x2 average-down fused with the truncation-error
 * estimate, and Kreiss-Oliger dissipation of order 2 and 3.
 *
 * Reference: source/kernels.h:18-42 (AverageDownWithTruncationError),
 *            :65-83 (KreissOligerDissipation<2>), :88-106 (<3>).
 *
 * AverageDownWithTruncationError(i,j,k) for each component n:
 *   c = sum of the 8 fine cells (2i..2i+1, 2j..2j+1, 2k..2k+1), taken in
 *       the order (0,0,0) (1,0,0) (0,1,0) (0,0,1) (1,1,0) (1,0,1) (0,1,1)
 *       (1,1,1);
 *   te(2i,2j,2k,n) = |crse(i,j,k,n) - c/8|;   crse(i,j,k,n) = c/8.
 * Kreiss-Oliger of order 2 adds  -sigma (D4x + D4y + D4z) / (16 dx)  and of
 * order 3 adds  +sigma (D6x + D6y + D6z) / (64 dx),  with D4 and D6 the
 * undivided 4th and 6th differences (binomial weights 1,-4,6 and
 * 1,-6,15,-20).
 */
#ifndef SLEDGEHAMR_KERNELS_H_
#define SLEDGEHAMR_KERNELS_H_

#include "sh_amrex.h"

namespace sledgehamr {
namespace kernels {

namespace detail {
/* Fine-cell visiting order of the 2x2x2 block. */
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr int oct_dx(int o) {
    return (o == 1 || o == 4 || o == 5 || o == 7) ? 1 : 0;
}
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr int oct_dy(int o) {
    return (o == 2 || o == 4 || o == 6 || o == 7) ? 1 : 0;
}
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE constexpr int oct_dz(int o) {
    return (o == 3 || o == 5 || o == 6 || o == 7) ? 1 : 0;
}
} // namespace detail

AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE void
AverageDownWithTruncationError(int i, int j, int k, const int ncomp,
                               amrex::Array4<double> const &crse,
                               amrex::Array4<double const> const &fine,
                               amrex::Array4<double> const &te) {
    const int fi = 2 * i, fj = 2 * j, fk = 2 * k;
    for (int n = 0; n < ncomp; ++n) {
        double sum = fine(fi, fj, fk, n);
        for (int o = 1; o < 8; ++o)
            sum += fine(fi + detail::oct_dx(o), fj + detail::oct_dy(o),
                        fk + detail::oct_dz(o), n);
        const double avg = 0.125 * sum;
        te(fi, fj, fk, n) = std::fabs(crse(i, j, k, n) - avg);
        crse(i, j, k, n) = avg;
    }
}

template <int Order>
AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double
KreissOligerDissipation(const amrex::Array4<double const> &state, const int i,
                        const int j, const int k, const int c, const double dx,
                        const double dissipation_strength) {
    static_assert(Order == 2 || Order == 3, "KO dissipation order 2 or 3");
    auto diff = [&](int ax) {
        auto f = [&](int d) {
            return ax == 0 ? state(i + d, j, k, c)
                           : (ax == 1 ? state(i, j + d, k, c)
                                      : state(i, j, k + d, c));
        };
        if constexpr (Order == 2) {
            double v = f(2);
            v -= 4. * f(1);
            v += f(-2);
            v -= 4. * f(-1);
            v += 6. * f(0);
            return v;
        } else {
            double v = f(3);
            v -= 6. * f(2);
            v += 15. * f(1);
            v += f(-3);
            v -= 6. * f(-2);
            v += 15. * f(-1);
            v -= 20. * f(0);
            return v;
        }
    };
    const double sum = diff(0) + diff(1) + diff(2);
    if constexpr (Order == 2)
        return -dissipation_strength * sum / 16. / dx;
    else
        return dissipation_strength * sum / 64. / dx;
}

} // namespace kernels
} // namespace sledgehamr

#endif // SLEDGEHAMR_KERNELS_H_
