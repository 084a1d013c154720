/* FirstOrderPhaseTransition equations of motion:
 *   Phi' = dPhi,   dPhi' = lap(Phi) + V'(Phi)
 * with V'(Phi) = q2 Phi + q3 Phi^2 + q4 Phi^3 (params[1..3]) for the pure
 * potential (params[0] = 0), or, for the piecewise potential (params[0] = 1),
 * that cubic below Phi = phiesc (params[6]) and -vareps^2 (Phi - vbar)
 * (params[5], params[4]) above it.  4th-order Laplacian.
 * GW source: u_ij' = du_ij,  du_ij' = lap(u_ij) + d_i Phi d_j Phi (4th-order
 * Laplacian and gradient).
 * Reference: projects/FirstOrderPhaseTransition/kernels_rhs.h:20-54 (Rhs),
 * :56-109 (GravitationalWavesRhs<true>).
 */
#ifndef SH_PROJECTS_FOPT_KERNELS_RHS_H_
#define SH_PROJECTS_FOPT_KERNELS_RHS_H_

#include <sledgehamr_utils.h>

#include "setup.h"

namespace FirstOrderPhaseTransition {

AMREX_GPU_DEVICE AMREX_FORCE_INLINE double PotentialGradient(const double phi,
                                                             const double *params) {
    const double q2 = params[1], q3 = params[2], q4 = params[3];
    const double cubic = q2 * phi + q3 * phi * phi + q4 * phi * phi * phi;
    if (static_cast<int>(params[0]) == PotentialType::Piecewise) {
        const double vbar = params[4], vareps = params[5], phiesc = params[6];
        const double below = phi < phiesc;
        return below * cubic - (1 - below) * vareps * vareps * (phi - vbar);
    }
    return cubic;
}

AMREX_GPU_DEVICE AMREX_FORCE_INLINE void
Rhs(const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, const int i,
    const int j, const int k, const int lev, const double time, const double dt,
    const double dx, const double *params) {
    const double phi = state(i, j, k, Scalar::Phi);
    rhs(i, j, k, Scalar::Phi) = state(i, j, k, Scalar::dPhi);
    rhs(i, j, k, Scalar::dPhi) =
        sledgehamr::utils::Laplacian<2>(state, i, j, k, Scalar::Phi, dx * dx) +
        PotentialGradient(phi, params);
}

template <>
AMREX_GPU_DEVICE AMREX_FORCE_INLINE void GravitationalWavesRhs<true>(
    const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, const int i,
    const int j, const int k, const int lev, const double time, const double dt,
    const double dx, const double *params) {
    constexpr int ax_a[6] = {0, 1, 2, 0, 0, 1};
    constexpr int ax_b[6] = {0, 1, 2, 1, 2, 2};
    double g[3];
    for (int ax = 0; ax < 3; ++ax)
        g[ax] = sledgehamr::utils::Gradient<2>(state, i, j, k, Scalar::Phi, dx, "xyz"[ax]);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        rhs(i, j, k, Gw::u_xx + q) = state(i, j, k, Gw::du_xx + q);
        rhs(i, j, k, Gw::du_xx + q) =
            sledgehamr::utils::Laplacian<2>(state, i, j, k, Gw::u_xx + q, dx * dx) +
            g[ax_a[q]] * g[ax_b[q]];
    }
}

} // namespace FirstOrderPhaseTransition

#endif
