/* FirstOrderPhaseTransition project: real scalar Phi with momentum dPhi
 * (projects/FirstOrderPhaseTransition/setup.h:8-11 of sledgehamr). */
#ifndef SH_PROJECTS_FOPT_SETUP_H_
#define SH_PROJECTS_FOPT_SETUP_H_

#include <sledgehamr.h>

namespace FirstOrderPhaseTransition {
SLEDGEHAMR_ADD_SCALARS(Phi)
SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(dPhi)
enum PotentialType { PureLambdaBar = 0, Piecewise = 1 };
} // namespace FirstOrderPhaseTransition

#endif
