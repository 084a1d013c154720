/* AxionStrings equations of motion in conformal time eta:
 *   Psi' = Pi,
 *   Pi'  = -2 Pi / eta + lap(Psi) - Psi [eta^2 (|Psi|^2 - 1) + 0.56233],
 * with the 4th-order (13-point) Laplacian.  The GW source hook evolves the
 * six tensor components u_ij with friction -2 du/eta and source
 * d_i Psi1 d_j Psi1 + d_i Psi2 d_j Psi2; like the reference it stores its
 * results in the u_* slots (first du, then the acceleration) and leaves the
 * du_* slots untouched.
 * Reference: projects/AxionStrings/kernels_rhs.h:21-49 (Rhs), :63-135 (GW).
 */
#ifndef SH_PROJECTS_AXION_STRINGS_KERNELS_RHS_H_
#define SH_PROJECTS_AXION_STRINGS_KERNELS_RHS_H_

#include <sledgehamr_utils.h>

#include "setup.h"

namespace AxionStrings {

AMREX_GPU_DEVICE AMREX_FORCE_INLINE void
Rhs(const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, const int i,
    const int j, const int k, const int lev, const double time, const double dt,
    const double dx, const double *params) {
    const double psi1 = state(i, j, k, Scalar::Psi1);
    const double psi2 = state(i, j, k, Scalar::Psi2);
    const double pi1 = state(i, j, k, Scalar::Pi1);
    const double pi2 = state(i, j, k, Scalar::Pi2);
    const double eta = time;
    const double friction = -2. / eta;
    const double lap1 = sledgehamr::utils::Laplacian<2>(state, i, j, k, Scalar::Psi1, dx * dx);
    const double lap2 = sledgehamr::utils::Laplacian<2>(state, i, j, k, Scalar::Psi2, dx * dx);
    const double v = eta * eta * (psi1 * psi1 + psi2 * psi2 - 1.) + 0.56233;
    rhs(i, j, k, Scalar::Psi1) = pi1;
    rhs(i, j, k, Scalar::Psi2) = pi2;
    rhs(i, j, k, Scalar::Pi1) = friction * pi1 + lap1 - psi1 * v;
    rhs(i, j, k, Scalar::Pi2) = friction * pi2 + lap2 - psi2 * v;
}

template <>
AMREX_GPU_DEVICE AMREX_FORCE_INLINE void GravitationalWavesRhs<true>(
    const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, const int i,
    const int j, const int k, const int lev, const double time, const double dt,
    const double dx, const double *params) {
    constexpr int ax_a[6] = {0, 1, 2, 0, 0, 1};
    constexpr int ax_b[6] = {0, 1, 2, 1, 2, 2};
    const double friction = -2. / time;
    double g1[3], g2[3];
    for (int ax = 0; ax < 3; ++ax) {
        g1[ax] = sledgehamr::utils::Gradient<2>(state, i, j, k, Scalar::Psi1, dx, "xyz"[ax]);
        g2[ax] = sledgehamr::utils::Gradient<2>(state, i, j, k, Scalar::Psi2, dx, "xyz"[ax]);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const double du = state(i, j, k, Gw::du_xx + q);
        rhs(i, j, k, Gw::u_xx + q) = du;
        rhs(i, j, k, Gw::u_xx + q) =
            friction * du + sledgehamr::utils::Laplacian<2>(state, i, j, k, Gw::u_xx + q, dx * dx) +
            g1[ax_a[q]] * g1[ax_b[q]] + g2[ax_a[q]] * g2[ax_b[q]];
    }
}

} // namespace AxionStrings

#endif
