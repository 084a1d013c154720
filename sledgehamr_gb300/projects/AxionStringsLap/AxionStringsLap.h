/* AxionStringsLap1/2/3: the axion-string equations with a selectable
 * Laplacian order, used by the 128^3 single-level and ensemble workloads
 * whose specification asks for the 2nd-order (7-point) Laplacian and a
 * plain quartic potential:
 *   Psi' = Pi,
 *   Pi'  = -2 Pi / eta + lap_N(Psi) - lambda Psi [eta^2 (|Psi|^2 - 1) + c]
 * with lambda = params[0] and c = params[1] (0 for the plain potential,
 * 0.56233 to reproduce NextToMinimalExample exactly for N = 2).
 * Tagging hooks are those of AxionStrings (string winding; dt-scaled
 * momentum truncation errors).
 * This is a project of this library; the reference has the N = 2 form as
 * projects/NextToMinimalExample/NextToMinimalExample.h:11-43.
 */
#ifndef SH_PROJECTS_AXION_STRINGS_LAP_H_
#define SH_PROJECTS_AXION_STRINGS_LAP_H_

#include <sledgehamr.h>

#include "../AxionStrings/string_winding.h"

#define SH_AXION_STRINGS_LAP_PROJECT(NS, ORDER)                                \
    namespace NS {                                                             \
    SLEDGEHAMR_ADD_SCALARS(Psi1, Psi2)                                         \
    SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(Pi1, Pi2)                                 \
    AMREX_GPU_DEVICE AMREX_FORCE_INLINE void                                   \
    Rhs(const amrex::Array4<double> &rhs, const amrex::Array4<const double> &state, \
        const int i, const int j, const int k, const int lev, const double time, \
        const double dt, const double dx, const double *params) {             \
        const double lambda = params[0], c = params[1];                        \
        const double psi1 = state(i, j, k, Scalar::Psi1);                      \
        const double psi2 = state(i, j, k, Scalar::Psi2);                      \
        const double pi1 = state(i, j, k, Scalar::Pi1);                        \
        const double pi2 = state(i, j, k, Scalar::Pi2);                        \
        const double eta = time;                                               \
        const double friction = -2. / eta;                                     \
        const double v = lambda * (eta * eta * (psi1 * psi1 + psi2 * psi2 - 1.) + c); \
        rhs(i, j, k, Scalar::Psi1) = pi1;                                      \
        rhs(i, j, k, Scalar::Psi2) = pi2;                                      \
        rhs(i, j, k, Scalar::Pi1) = friction * pi1 +                           \
            sledgehamr::utils::Laplacian<ORDER>(state, i, j, k, Scalar::Psi1, dx * dx) - \
            psi1 * v;                                                          \
        rhs(i, j, k, Scalar::Pi2) = friction * pi2 +                           \
            sledgehamr::utils::Laplacian<ORDER>(state, i, j, k, Scalar::Psi2, dx * dx) - \
            psi2 * v;                                                          \
    }                                                                          \
    SH_AXION_STRING_TAGGING                                                    \
    SLEDGEHAMR_FINISH_SETUP                                                    \
    }

SH_AXION_STRINGS_LAP_PROJECT(AxionStringsLap1, 1)
SH_AXION_STRINGS_LAP_PROJECT(AxionStringsLap2, 2)
SH_AXION_STRINGS_LAP_PROJECT(AxionStringsLap3, 3)

#endif
