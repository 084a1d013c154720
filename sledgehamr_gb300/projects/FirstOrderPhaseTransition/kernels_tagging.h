/* FirstOrderPhaseTransition truncation-error modifiers: the error of each
 * component is divided by the maximum of |component| (params[n], filled by
 * the host from the level norms), and for momenta (dPhi, du_*) multiplied by
 * dt first.  No user tagging criterion.
 * Reference: projects/FirstOrderPhaseTransition/kernels_tagging.h:13-45.
 */
#ifndef SH_PROJECTS_FOPT_KERNELS_TAGGING_H_
#define SH_PROJECTS_FOPT_KERNELS_TAGGING_H_

#include "setup.h"

namespace FirstOrderPhaseTransition {

#define SH_FOPT_TE_SCALED(c, factor)                                           \
    template <>                                                                \
    AMREX_GPU_HOST_DEVICE AMREX_FORCE_INLINE double TruncationModifier<c>(     \
        const amrex::Array4<const double> &state, const int i, const int j,    \
        const int k, const int lev, const double time, const double dt,        \
        const double dx, const double truncation_error, const double *params) { \
        return truncation_error * factor / params[c];                          \
    }
SH_FOPT_TE_SCALED(Scalar::Phi, 1.)
SH_FOPT_TE_SCALED(Gw::u_xx, 1.)
SH_FOPT_TE_SCALED(Gw::u_yy, 1.)
SH_FOPT_TE_SCALED(Gw::u_zz, 1.)
SH_FOPT_TE_SCALED(Gw::u_xy, 1.)
SH_FOPT_TE_SCALED(Gw::u_xz, 1.)
SH_FOPT_TE_SCALED(Gw::u_yz, 1.)
SH_FOPT_TE_SCALED(Scalar::dPhi, dt)
SH_FOPT_TE_SCALED(Gw::du_xx, dt)
SH_FOPT_TE_SCALED(Gw::du_yy, dt)
SH_FOPT_TE_SCALED(Gw::du_zz, dt)
SH_FOPT_TE_SCALED(Gw::du_xy, dt)
SH_FOPT_TE_SCALED(Gw::du_xz, dt)
SH_FOPT_TE_SCALED(Gw::du_yz, dt)
#undef SH_FOPT_TE_SCALED

} // namespace FirstOrderPhaseTransition

#endif
