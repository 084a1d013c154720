/* A project added to the library without editing it: its hooks (a damped
 * wave equation phi'' = lap phi - 0.1 phi', written the way sledgehamr
 * projects are) and one SH_DEFINE_PROJECT line, compiled into an object
 * and linked with the library's own objects by tests/test_project_registry.py. */
#include <sledgehamr.h>

namespace WaveTest {

SLEDGEHAMR_ADD_SCALARS(Phi)
SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(dPhi)

AMREX_GPU_DEVICE AMREX_FORCE_INLINE void
Rhs(const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, const int i,
    const int j, const int k, const int lev, const double time, const double dt,
    const double dx, const double *params) {
    rhs(i, j, k, Scalar::Phi) = state(i, j, k, Scalar::dPhi);
    rhs(i, j, k, Scalar::dPhi) =
        sledgehamr::utils::Laplacian<1>(state, i, j, k, Scalar::Phi, dx * dx) -
        0.1 * state(i, j, k, Scalar::dPhi);
}

SLEDGEHAMR_FINISH_SETUP

} // namespace WaveTest

#include "sh_stage.cuh"
SH_DEFINE_PROJECT(WaveTest, ::WaveTest, false, 1)
