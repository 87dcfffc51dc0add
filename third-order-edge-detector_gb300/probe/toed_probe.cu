// toed_probe.cu -- FP32 / FP64 issue-rate probe (toed_peak_probe), a
// measurement tool of bench.py built into its own small library
// (libtoed_probe.so), not part of the detector's C ABI.
//
// The detection path is bound by FP32 FMA issue, not by HBM or tensor
// cores, so its roofline denominator is the FP32 FMA rate at the clocks of
// the run.  Each thread keeps 8 independent FMA chains in registers (no
// memory traffic inside the loop) on a grid of 4 CTAs x 256 threads per SM.
#include <cuda_runtime.h>

#include "../../include/toed_gb300.h"

// kind 0: FP32, 1: FP64; *tflops gets the sustained FMA rate of `iters`
// iterations on all SMs (CUDA events on `stream`).
extern "C" toed_status toed_peak_probe(int kind, int iters, cudaStream_t stream, double* tflops);

namespace {
template <typename T>
__global__ void __launch_bounds__(256) fma_loop(int iters, T seed, T* sink)
{
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + (T)(threadIdx.x + k);
    const T m = (T)0.9999, c = (T)1e-7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = a[k] * m + c;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == (T)-1) sink[threadIdx.x] = s;  // keeps the loop alive; never true
}
}  // namespace

extern "C" toed_status toed_peak_probe(int kind, int iters, cudaStream_t stream, double* tflops)
{
    if (!tflops || iters <= 0 || (kind != 0 && kind != 1)) return TOED_ERR_INVALID_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TOED_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return TOED_ERR_CUDA;
    void* sink = nullptr;
    if (cudaMalloc(&sink, 256 * sizeof(double)) != cudaSuccess) return TOED_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const dim3 grid(4 * sms), block(256);
    // warm-up, then the timed launch
    if (kind == 0) {
        fma_loop<float><<<grid, block, 0, stream>>>(iters / 4 + 1, 1.0f, (float*)sink);
        cudaEventRecord(e0, stream);
        fma_loop<float><<<grid, block, 0, stream>>>(iters, 1.0f, (float*)sink);
    } else {
        fma_loop<double><<<grid, block, 0, stream>>>(iters / 4 + 1, 1.0, (double*)sink);
        cudaEventRecord(e0, stream);
        fma_loop<double><<<grid, block, 0, stream>>>(iters, 1.0, (double*)sink);
    }
    cudaEventRecord(e1, stream);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess || ms <= 0.f) return TOED_ERR_CUDA;
    const double flops = 2.0 * 8.0 * (double)iters * grid.x * block.x;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return TOED_OK;
}
