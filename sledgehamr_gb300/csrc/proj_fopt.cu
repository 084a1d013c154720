/* FirstOrderPhaseTransition project kernels (hooks in
 * projects/FirstOrderPhaseTransition). */
#include "../projects/FirstOrderPhaseTransition/setup.h"
#include "../projects/FirstOrderPhaseTransition/kernels_rhs.h"
#include "../projects/FirstOrderPhaseTransition/kernels_tagging.h"
namespace FirstOrderPhaseTransition {
SLEDGEHAMR_FINISH_SETUP
}
#include "sh_stage.cuh"
SH_DEFINE_PROJECT(FirstOrderPhaseTransition, ::FirstOrderPhaseTransition, true, 2)
