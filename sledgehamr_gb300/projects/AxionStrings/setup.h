/* AxionStrings project: complex scalar Psi = Psi1 + i Psi2 with conjugate
 * momenta Pi1, Pi2 (projects/AxionStrings/setup.h:6-7 of sledgehamr). */
#ifndef SH_PROJECTS_AXION_STRINGS_SETUP_H_
#define SH_PROJECTS_AXION_STRINGS_SETUP_H_

#include <sledgehamr.h>

namespace AxionStrings {
SLEDGEHAMR_ADD_SCALARS(Psi1, Psi2)
SLEDGEHAMR_ADD_CONJUGATE_MOMENTA(Pi1, Pi2)
} // namespace AxionStrings

#endif
