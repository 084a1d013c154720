/* Per-cell output functions of the projects (device side), evaluated with
 * separately rounded operations so that the values equal a CPU evaluation
 * bit for bit.  Components of the AxionStrings layout Psi1 Psi2 Pi1 Pi2
 * (0..3) or one component `comp`, at stride `stride` from v:
 *   SH_OUT_COMPONENT     state(comp)
 *   SH_OUT_COMPONENT_SQ  state(comp)^2  (FirstOrderPhaseTransition dPhi2,
 *                        projects/FirstOrderPhaseTransition/kernels_misc.h:10-18)
 *   SH_OUT_A_PRIME2      ((Psi1 Pi2 - Psi2 Pi1) / r^2)^2, r^2 = Psi1^2 + Psi2^2
 *                        (projects/AxionStrings/kernels_energy_densities.h:21-33,
 *                        NextToMinimalExample a_dot_sq)
 *   SH_OUT_A_PRIME_SCREENED  Psi1 Pi2 - Psi2 Pi1 (kernels_energy_densities.h:48-58)
 *   SH_OUT_R_PRIME2      (Psi1 Pi1 + Psi2 Pi2)^2 / r^2 (kernels_energy_densities.h:73-85) */
#ifndef SH_OUT_CUH_
#define SH_OUT_CUH_

#include "sledgehamr_gb300.h"

namespace sh {

__device__ __forceinline__ double out_function(int fn, int comp, const double *v,
                                               long long stride) {
    if (fn == SH_OUT_COMPONENT) return v[comp * stride];
    if (fn == SH_OUT_COMPONENT_SQ) return __dmul_rn(v[comp * stride], v[comp * stride]);
    const double Psi1 = v[0], Psi2 = v[stride], Pi1 = v[2 * stride], Pi2 = v[3 * stride];
    if (fn == SH_OUT_A_PRIME_SCREENED) return __dsub_rn(__dmul_rn(Psi1, Pi2), __dmul_rn(Psi2, Pi1));
    const double r2 = __dadd_rn(__dmul_rn(Psi1, Psi1), __dmul_rn(Psi2, Psi2));
    if (fn == SH_OUT_A_PRIME2) {
        const double pa =
            __ddiv_rn(__dsub_rn(__dmul_rn(Psi1, Pi2), __dmul_rn(Psi2, Pi1)), r2);
        return __dmul_rn(pa, pa);
    }
    const double pr = __dadd_rn(__dmul_rn(Psi1, Pi1), __dmul_rn(Psi2, Pi2));
    return __ddiv_rn(__dmul_rn(pr, pr), r2);
}

} // namespace sh

#endif
