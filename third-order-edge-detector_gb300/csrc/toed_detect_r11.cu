// Detection kernels for half-width r = 11.
#include "toed_detect_inst.cuh"
TOED_DETECT_INSTANCE(11)
