// Detection kernels for half-width r = 4.
#include "toed_detect_inst.cuh"
TOED_DETECT_INSTANCE(4)
