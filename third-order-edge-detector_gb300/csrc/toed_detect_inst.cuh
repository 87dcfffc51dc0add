// toed_detect_inst.cuh -- one translation unit per kernel radius keeps the
// heavily unrolled instantiations compiling in parallel.
#pragma once
#include "toed_detect.cuh"
#include "toed_internal.h"

#define TOED_DETECT_INSTANCE(R)                                                    \
    namespace toed {                                                               \
    DetectEntry detect_entry_r##R(bool hyb)                                        \
    {                                                                              \
        DetectEntry e;                                                             \
        e.smem = Cfg<R>::smem;                                                     \
        e.func = hyb ? (const void*)toed_detect_kernel<R, true>                    \
                     : (const void*)toed_detect_kernel<R, false>;                  \
        return e;                                                                  \
    }                                                                              \
    }
