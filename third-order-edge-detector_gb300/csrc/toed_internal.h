// toed_internal.h -- declarations shared between the kernel translation units
// and the host implementation of the C ABI (not part of the public ABI).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace toed {

struct BatchParams;

// One compiled detection kernel: entry point and its dynamic shared memory.
struct DetectEntry {
    const void* func;
    size_t smem;
};

// Per-radius instantiations (toed_detect_r<R>.cu); hyb selects the FP64 epilogue.
DetectEntry detect_entry(int radius, bool hyb);

cudaError_t launch_finalize(const BatchParams& p, cudaStream_t stream);

}  // namespace toed
