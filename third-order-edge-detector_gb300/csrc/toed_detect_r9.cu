// Detection kernels for half-width r = 9.
#include "toed_detect_inst.cuh"
TOED_DETECT_INSTANCE(9)
