// The persistent, batched geocode kernel: the device code of gslc_kernels.cu
// compiled as its own translation unit with only the persistent launchers.
#define GSLC_PERSISTENT_TU 1
#include "gslc_kernels.cu"
