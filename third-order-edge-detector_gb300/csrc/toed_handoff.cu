// toed_handoff.cu -- what the reference's drivers do with the edgel list
// after detection: the column-major double array that curvelet formation
// reads (form_curvelet_process, fed by main_cpu_DP.cpp:225-236), and the
// tab-separated text files non_maximum_suppresion writes
// (cpu_toed.cpp:556-580 with the stream's default 6 significant digits,
// gpu_toed.hpp:452-478 with 10).
#include <cstdio>

#include "toed_common.cuh"

namespace toed {
namespace {

// Column j of the n x 4 row-major list -> out[j * n + i] (coalesced writes).
__global__ void edgels_to_columns(const void* __restrict__ e, int f64, int n, double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (f64) {
        const double4_32a v = reinterpret_cast<const double4_32a*>(e)[i];
        out[i] = v.x;
        out[n + i] = v.y;
        out[2LL * n + i] = v.z;
        out[3LL * n + i] = v.w;
    } else {
        const float4 v = reinterpret_cast<const float4*>(e)[i];
        out[i] = v.x;
        out[n + i] = v.y;
        out[2LL * n + i] = v.z;
        out[3LL * n + i] = v.w;
    }
}

}  // namespace
}  // namespace toed

extern "C" toed_status toed_edgels_to_columns(const void* edgels, int dtype, int n, double* columns,
                                              cudaStream_t stream)
{
    if (n < 0 || (n > 0 && (!edgels || !columns))) return TOED_ERR_INVALID_ARG;
    if (dtype != TOED_F32 && dtype != TOED_F64) return TOED_ERR_INVALID_ARG;
    if (reinterpret_cast<uintptr_t>(edgels) % (dtype == TOED_F64 ? 32 : 16) != 0) return TOED_ERR_INVALID_ARG;
    if (n == 0) return TOED_OK;
    toed::edgels_to_columns<<<(n + 255) / 256, 256, 0, stream>>>(edgels, dtype == TOED_F64, n, columns);
    return cudaGetLastError() == cudaSuccess ? TOED_OK : TOED_ERR_CUDA;
}

extern "C" toed_status toed_write_edgels_txt(const char* path, const void* edgels, int dtype, int n, int precision)
{
    if (!path || n < 0 || (n > 0 && !edgels) || precision < 1 || precision > 17) return TOED_ERR_INVALID_ARG;
    if (dtype != TOED_F32 && dtype != TOED_F64) return TOED_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "w");
    if (!f) return TOED_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < 4; ++j) {
            const double v = dtype == TOED_F64 ? static_cast<const double*>(edgels)[4LL * i + j]
                                               : (double)static_cast<const float*>(edgels)[4LL * i + j];
            std::fprintf(f, "%.*g\t", precision, v);
        }
        std::fputc('\n', f);
    }
    return std::fclose(f) == 0 ? TOED_OK : TOED_ERR_INVALID_ARG;
}
