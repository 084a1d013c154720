/* AxionStringsLap1/2/3 project kernels (projects/AxionStringsLap). */
#include "../projects/AxionStringsLap/AxionStringsLap.h"
#include "sh_stage.cuh"
SH_DEFINE_PROJECT(AxionStringsLap1, ::AxionStringsLap1, false, 1)
SH_DEFINE_PROJECT(AxionStringsLap2, ::AxionStringsLap2, false, 2)
SH_DEFINE_PROJECT(AxionStringsLap3, ::AxionStringsLap3, false, 3)
