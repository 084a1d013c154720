/* AxionStrings project kernels (hooks in projects/AxionStrings). */
#include "../projects/AxionStrings/setup.h"
#include "../projects/AxionStrings/kernels_rhs.h"
#include "../projects/AxionStrings/kernels_tagging.h"
namespace AxionStrings {
SLEDGEHAMR_FINISH_SETUP
}
#include "sh_stage.cuh"
SH_DEFINE_PROJECT(AxionStrings, ::AxionStrings, true, 2)
