// toed_detect_inst.cuh -- one translation unit per kernel radius keeps the
// heavily unrolled instantiations compiling in parallel.
#pragma once
#include "toed_detect.cuh"
#include "toed_internal.h"

#define TOED_DETECT_INSTANCE(R)                                                    \
    namespace toed {                                                               \
    DetectEntry detect_entry_r##R(bool hyb, bool async, bool nmsto)                \
    {                                                                              \
        DetectEntry e;                                                             \
        e.smem = Cfg<R>::smem;                                                     \
        if (nmsto)                                                                 \
            e.func = hyb ? (const void*)toed_detect_kernel<R, true, false, true>   \
                         : (const void*)toed_detect_kernel<R, false, false, true>; \
        else if (async)                                                            \
            e.func = hyb ? (const void*)toed_detect_kernel<R, true, true>          \
                         : (const void*)toed_detect_kernel<R, false, true>;        \
        else                                                                       \
            e.func = hyb ? (const void*)toed_detect_kernel<R, true, false>         \
                         : (const void*)toed_detect_kernel<R, false, false>;       \
        return e;                                                                  \
    }                                                                              \
    }
