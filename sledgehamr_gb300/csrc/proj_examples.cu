/* MinimalExample and NextToMinimalExample project kernels. */
#include "../projects/MinimalExample/MinimalExample.h"
#include "../projects/NextToMinimalExample/NextToMinimalExample.h"
#include "sh_stage.cuh"
SH_DEFINE_PROJECT(MinimalExample, ::MinimalExample, false, 2)
SH_DEFINE_PROJECT(NextToMinimalExample, ::NextToMinimalExample, false, 2)
