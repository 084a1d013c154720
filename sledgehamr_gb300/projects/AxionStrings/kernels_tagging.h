/* AxionStrings refinement criteria: string winding tags and truncation
 * errors of Pi1, Pi2, du_* multiplied by dt before the comparison with the
 * threshold (see string_winding.h).
 * Reference: projects/AxionStrings/kernels_tagging.h:16-131.
 */
#ifndef SH_PROJECTS_AXION_STRINGS_KERNELS_TAGGING_H_
#define SH_PROJECTS_AXION_STRINGS_KERNELS_TAGGING_H_

#include "setup.h"
#include "string_winding.h"

namespace AxionStrings {
SH_AXION_STRING_TAGGING
} // namespace AxionStrings

#endif
