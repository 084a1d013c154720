/* NextToMinimalExample project: the MinimalExample equations with the
 * potential term scaled by lambda = params[0], which the project class hands
 * to the kernels through SetParamsRhs.
 * Reference: projects/NextToMinimalExample/NextToMinimalExample.h:11-43, :82-85.
 */
#ifndef SH_PROJECTS_NEXT_TO_MINIMAL_EXAMPLE_H_
#define SH_PROJECTS_NEXT_TO_MINIMAL_EXAMPLE_H_

#include <sledgehamr.h>

namespace NextToMinimalExample {

SLEDGEHAMR_ADD_SCALARS(Psi1, Psi2)
SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(Pi1, Pi2)

AMREX_GPU_DEVICE AMREX_FORCE_INLINE void
Rhs(const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, const int i,
    const int j, const int k, const int lev, const double time, const double dt,
    const double dx, const double *params) {
    const double lambda = params[0];
    const double psi1 = state(i, j, k, Scalar::Psi1), psi2 = state(i, j, k, Scalar::Psi2);
    const double pi1 = state(i, j, k, Scalar::Pi1), pi2 = state(i, j, k, Scalar::Pi2);
    const double eta = time;
    const double friction = -2. / eta;
    const double v = lambda * (eta * eta * (psi1 * psi1 + psi2 * psi2 - 1.) + 0.56233);
    rhs(i, j, k, Scalar::Psi1) = pi1;
    rhs(i, j, k, Scalar::Psi2) = pi2;
    rhs(i, j, k, Scalar::Pi1) = friction * pi1 +
        sledgehamr::utils::Laplacian<2>(state, i, j, k, Scalar::Psi1, dx * dx) - psi1 * v;
    rhs(i, j, k, Scalar::Pi2) = friction * pi2 +
        sledgehamr::utils::Laplacian<2>(state, i, j, k, Scalar::Psi2, dx * dx) - psi2 * v;
}

SLEDGEHAMR_FINISH_SETUP

class NextToMinimalExample : public sledgehamr::Sledgehamr {
  public:
    SLEDGEHAMR_INITIALIZE_PROJECT(NextToMinimalExample)
    void SetParamsRhs(std::vector<double> &params, const double time,
                      const int lev) override {
        params.push_back(lambda);
    }
    double lambda = 1.;
};

} // namespace NextToMinimalExample

#endif
