// toed_internal.h -- declarations shared between the kernel translation units
// and the host implementation of the C ABI (not part of the public ABI).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "toed_common.cuh"

namespace toed {

// One compiled detection kernel: entry point and its dynamic shared memory.
struct DetectEntry {
    const void* func;
    size_t smem;
};

// Per-radius instantiations (toed_detect_r<R>.cu); hyb selects the FP64
// epilogue, async the variant that stages rows by per-thread async copies,
// nmsto the corrected-normal NMS (rows by TMA or plain loads).
DetectEntry detect_entry(int radius, bool hyb, bool async = false, bool nmsto = false);

cudaError_t launch_finalize(const BatchParams& p, cudaStream_t stream);
// Load the ordering pass' kernels for `radius` (and the QaD variant) now:
// with lazy module loading a kernel's first launch may wait for the device,
// which must not happen while a detection launch waits for copies that the
// host has yet to enqueue.
cudaError_t preload_finalize(int radius, bool qad);
// The ordering pass's last kernel in the TOED_ORI_QAD orientation mode (toed_qad.cu).
cudaError_t launch_scatter_qad(const BatchParams& p, cudaStream_t stream);
cudaError_t preload_scatter_qad(int radius);

// Host-side checks of one device image (pointers, sizes, dtype, the
// 16-byte edgel and 4-byte float32 pixel alignment): TOED_OK or the status
// every detection entry point returns for it.
toed_status check_image(const toed_image& im);

// Fill d.tma / d.tma_align / d.tma_boxw and encode the image's row map for
// TMA staging (kStepRows-row boxes, zero fill outside the image).  Leaves
// d.tma = 0 -- plain loads -- when the driver entry point is unavailable or
// the image's base or pitch is not 16-byte aligned.
void encode_rows_map(CUtensorMap* m, DetImage& d, int radius);

// Enqueue the adjoint (toed_backward.cu): clears each item's grad_pixels,
// then one kernel; dL/dsigma is added into *gsig.
cudaError_t backward_launch(const toed_grad_image* items, int n, const toed_params* prm, int r, double* gsig,
                            cudaStream_t stream);

// Scratch of the TO-correction pipeline (owned by the caller's context).
struct SubScratch {
    Scratch sc;
    float2* dir;          // per pixel
    int* eid;             // per pixel
    int* win;             // per pixel (dense maps)
    int* img_count;       // per map
    unsigned char* keep;  // per staged edgel
    double* work;         // interp_n > 0: resized maps (and orientations), per work pixel
};

// Enqueue the TO-correction kernels for up to kBatchMax maps (toed_subpix.cu).
cudaError_t subpix_launch(const toed_edgemap* maps, int n, const toed_subpix_params* prm, int r,
                          const SubScratch& s, cudaStream_t stream);

}  // namespace toed
