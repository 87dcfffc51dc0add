// toed_planes.cu -- the reference's dense two-kernel form behind the C ABI
// (toed_convolve_planes / toed_nms_planes), for callers that bind
// gpu_convolve / gpu_nms (gpu_kernels.hpp:24-63) and want the 2x-grid planes
// themselves.  The fused path (toed_detect) never materialises these planes;
// this one does, in FP32 or end-to-end FP64.
//
// planes_kernel : one CTA per 32x8 tile of original pixels; separable row
//                 pass of the 12 filter responses into shared memory, then
//                 one thread per original pixel evaluates the nine
//                 derivatives at its four sub-grids (cpu_toed.cpp:204-355),
//                 |grad I| and the TO orientation.
// direct_planes_kernel : the same planes with the reference's full 2-D
//                 window per derivative (toed_convolve_planes_direct).
// nms_kernel    : one thread per 2x-grid point, subpixel NMS as
//                 cpu_toed.cpp:399-495, writing the position maps.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {
void make_taps(double sigma, int r, TapBlock* tb);

namespace {
constexpr int TW = 32, TH = 8;

template <typename T>
struct TapsT {
    T v[8][kMaxTaps];
};

template <typename T>
__device__ __forceinline__ T load_pixel(const void* src, long long pitch, int H, int W, int dtype, int y, int x)
{
    if ((unsigned)y >= (unsigned)H || (unsigned)x >= (unsigned)W) return T(0);
    const long long o = (long long)y * pitch + x;
    if (dtype == TOED_U8) return (T)((const unsigned char*)src)[o];
    if (dtype == TOED_F32) return (T)((const float*)src)[o];
    return (T)((const double*)src)[o];
}

template <typename T>
__device__ __forceinline__ T to_orient(T fx, T fy, T fxx, T fxy, T fyy, T fxxy, T fxyy, T fxxx, T fyyy)
{
    T tix = fx * (T(2) * fxx * fxx + T(2) * fxy * fxy) + fy * (T(2) * fxx * fxy + T(2) * fyy * fxy) +
            T(2) * fx * fy * fxxy + fy * fy * fxyy + fx * fx * fxxx;
    T tiy = fx * (T(2) * fxx * fxy + T(2) * fyy * fxy) + fy * (T(2) * fyy * fyy + T(2) * fxy * fxy) +
            T(2) * fx * fy * fxyy + fx * fx * fxxy + fy * fy * fyyy;
    const T m = sqrt(tix * tix + tiy * tiy);
    tix /= m;
    tiy /= m;
    return atan2(tix, -tiy);
}

// Row-pass plane index: variant (0 T, 1 F, 2 S) x filter (0 G .. 3 Gxxx)
template <typename T>
__global__ void __launch_bounds__(256) planes_kernel(const void* src, int dtype, int H, int W, long long pitch,
                                                     int R, const __grid_constant__ TapsT<T> tp, T* Ix,
                                                     T* Iy, T* mag, T* ori)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sh = reinterpret_cast<T*>(smem_raw);
    const int NR = TH + 2 * R + 2, NIN = TW + 2 * R + 2;
    T* sIn = sh;                      // [NR][NIN]
    T* sRow = sh + NR * NIN;          // [12][NR][TW]
    const int i0 = blockIdx.y * TH, j0 = blockIdx.x * TW;
    for (int t = threadIdx.x; t < NR * NIN; t += blockDim.x) {
        const int rr = t / NIN, cc = t - rr * NIN;
        sIn[t] = load_pixel<T>(src, pitch, H, W, dtype, i0 - R - 1 + rr, j0 - R - 1 + cc);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < NR * TW; t += blockDim.x) {
        const int rr = t / TW, x = t - rr * TW;
        const T* v = sIn + rr * NIN + x;  // v[c] <-> image col j0 + x - (R+1) + c; centre c = R+1
        for (int f = 0; f < 4; ++f) {
            T tr = 0, sv = 0;
            for (int q = -R; q <= R; ++q) tr += v[R + 1 - q] * tp.v[f][q + R + 1];
            const T fu = tr + v[0] * tp.v[f][2 * R + 2] + v[2 * R + 2] * tp.v[f][0];
            for (int q = -(R + 1); q <= R + 1; ++q) sv += v[R + 1 - q] * tp.v[4 + f][q + R + 1];
            sRow[((0 * 4 + f) * NR + rr) * TW + x] = tr;
            sRow[((1 * 4 + f) * NR + rr) * TW + x] = fu;
            sRow[((2 * 4 + f) * NR + rr) * TW + x] = sv;
        }
    }
    __syncthreads();
    const int x = threadIdx.x % TW, yy = threadIdx.x / TW;
    const int i = i0 + yy, j = j0 + x;
    if (i >= H || j >= W) return;
    const int W2 = 2 * W;
    for (int sg = 0; sg < 4; ++sg) {
        const int a = sg >> 1, b = sg & 1;
        const int xv = b ? 2 : (a ? 1 : 0);
        const int yf = a ? 4 : 0;
        const int plo = (sg == 0) ? -R : -(R + 1), phi = (sg == 0) ? R : R + 1;
        const T* P0 = sRow + (xv * 4 + 0) * NR * TW + x;
        const T* P1 = sRow + (xv * 4 + 1) * NR * TW + x;
        const T* P2 = sRow + (xv * 4 + 2) * NR * TW + x;
        const T* P3 = sRow + (xv * 4 + 3) * NR * TW + x;
        T d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int p = plo; p <= phi; ++p) {
            const int row = yy + R + 1 - p;
            const T hG = P0[row * TW], hGx = P1[row * TW], hGxx = P2[row * TW], hGxxx = P3[row * TW];
            const T yG = tp.v[yf + 0][p + R + 1], yGx = tp.v[yf + 1][p + R + 1];
            const T yGxx = tp.v[yf + 2][p + R + 1], yGxxx = tp.v[yf + 3][p + R + 1];
            d[0] += hGx * yG;    // fx
            d[1] += hG * yGx;    // fy
            d[2] += hGxx * yG;   // fxx
            d[3] += hGx * yGx;   // fxy
            d[4] += hG * yGxx;   // fyy
            d[5] += hGxx * yGx;  // fxxy
            d[6] += hGx * yGxx;  // fxyy
            d[7] += hGxxx * yG;  // fxxx
            d[8] += hG * yGxxx;  // fyyy
        }
        const long long o = (long long)(2 * i + a) * W2 + (2 * j + b);
        Ix[o] = d[0];
        Iy[o] = d[1];
        mag[o] = sqrt(d[0] * d[0] + d[1] * d[1]);
        ori[o] = to_orient<T>(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) nms_kernel(int H2, int W2, const T* Ix, const T* Iy, const T* M, T thr,
                                                  int border, T* px, T* py)
{
    const long long n = (long long)H2 * W2;
    for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n;
         o += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(o / W2), j = (int)(o - (long long)i * W2);
        T ox = 0, oy = 0;
        if (i >= border && i < H2 - border && j >= border && j < W2 - border) {
            const T m = M[o], gx = Ix[o], gy = Iy[o];
            if (m > thr && !(fabs(gx) < T(10e-6) && fabs(gy) < T(10e-6))) {
                const T nx = gx / m, ny = gy / m;
                const bool xmaj = fabs(gx) >= fabs(gy);
                const int sx = gx >= 0 ? 1 : -1, sy = gy >= 0 ? 1 : -1;
                const T slope = xmaj ? fabs(ny) / fabs(nx) : fabs(nx) / fabs(ny);
                const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
                const T fp = M[(long long)(i + ar) * W2 + j + ac] * (1 - slope) + M[(long long)(i + sy) * W2 + j + sx] * slope;
                const T fm = M[(long long)(i - ar) * W2 + j - ac] * (1 - slope) + M[(long long)(i - sy) * W2 + j - sx] * slope;
                const T s = sqrt(1 + slope * slope);
                if ((m > fm && m >= fp) || (m >= fm && m > fp)) {
                    const T A = (fm + fp - 2 * m) / (2 * s * s);
                    const T B = (fp - fm) / (2 * s);
                    const T ss = -B / (2 * A);
                    if (fabs(ss) <= (T)1.4142135623730951) {
                        ox = j + ss * nx;
                        oy = i + ss * ny;
                    }
                }
            }
        }
        px[o] = ox;
        py[o] = oy;
    }
}

// The reference's own structure (gpu_convolve.cu:96-300): every derivative
// of every sub-grid a full 2-D window sum -- (2r+1)^2 taps on sub-grid (0,0),
// (2r+3)^2 on the others -- over a shared-memory tile, one thread per
// original pixel, row offset p outer and column offset q inner, each term
// the pixel times its x tap times its y tap.  The four column-tap products
// of a pixel are shared by the nine derivatives (4 multiplies + 9 FMAs per
// window tap).  Written with the window width as a template argument so the
// inner loop unrolls like the reference's fixed-size one.
constexpr int DTW = 16, DTH = 16;

template <typename T, int R>
__global__ void __launch_bounds__(DTW * DTH) direct_planes_kernel(const void* src, int dtype, int H, int W,
                                                                  long long pitch, const __grid_constant__ TapsT<T> tp,
                                                                  T* Ix, T* Iy, T* mag, T* ori)
{
    constexpr int NIN = DTW + 2 * R + 2, NR = DTH + 2 * R + 2;
    __shared__ T sIn[NR][NIN];
    const int i0 = blockIdx.y * DTH, j0 = blockIdx.x * DTW;
    for (int t = threadIdx.x; t < NR * NIN; t += DTW * DTH) {
        const int rr = t / NIN, cc = t - rr * NIN;
        sIn[rr][cc] = load_pixel<T>(src, pitch, H, W, dtype, i0 - R - 1 + rr, j0 - R - 1 + cc);
    }
    __syncthreads();
    const int x = threadIdx.x % DTW, y = threadIdx.x / DTW;
    const int i = i0 + y, j = j0 + x;
    if (i >= H || j >= W) return;
    const int W2 = 2 * W;
#pragma unroll 1
    for (int sg = 0; sg < 4; ++sg) {
        const int a = sg >> 1, b = sg & 1;
        const int h = sg ? R + 1 : R;  // window half-width
        const T* X = tp.v[b ? 4 : 0];  // filter f, tap k: X[f * kMaxTaps + k]
        const T* Y = tp.v[a ? 4 : 0];
        T d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll 1
        for (int p = -h; p <= h; ++p) {
            const T* row = &sIn[y + R + 1 - p][x + R + 1];  // row[-q]: pixel (i - p, j - q)
            const int kp = p + R + 1;
            const T yG = Y[kp], yGx = Y[kMaxTaps + kp], yGxx = Y[2 * kMaxTaps + kp], yGxxx = Y[3 * kMaxTaps + kp];
#pragma unroll
            for (int q = -(R + 1); q <= R + 1; ++q) {
                if (q < -h || q > h) continue;
                const int kq = q + R + 1;
                const T v = row[-q];
                const T vG = v * X[kq], vGx = v * X[kMaxTaps + kq], vGxx = v * X[2 * kMaxTaps + kq],
                        vGxxx = v * X[3 * kMaxTaps + kq];
                d[0] += vGx * yG;    // fx
                d[1] += vG * yGx;    // fy
                d[2] += vGxx * yG;   // fxx
                d[3] += vGx * yGx;   // fxy
                d[4] += vG * yGxx;   // fyy
                d[5] += vGxx * yGx;  // fxxy
                d[6] += vGx * yGxx;  // fxyy
                d[7] += vGxxx * yG;  // fxxx
                d[8] += vG * yGxxx;  // fyyy
            }
        }
        const long long o = (long long)(2 * i + a) * W2 + (2 * j + b);
        Ix[o] = d[0];
        Iy[o] = d[1];
        mag[o] = sqrt(d[0] * d[0] + d[1] * d[1]);
        ori[o] = to_orient<T>(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]);
    }
}

template <typename T, int R>
cudaError_t launch_direct(const void* pixels, int dtype, int h, int w, int pitch, const TapsT<T>& tt, void* Ix,
                          void* Iy, void* gm, void* orient, cudaStream_t stream)
{
    dim3 grid((w + DTW - 1) / DTW, (h + DTH - 1) / DTH);
    direct_planes_kernel<T, R><<<grid, DTW * DTH, 0, stream>>>(pixels, dtype, h, w, (long long)pitch, tt, (T*)Ix,
                                                               (T*)Iy, (T*)gm, (T*)orient);
    return cudaGetLastError();
}

template <typename T>
cudaError_t run_direct(const void* pixels, int dtype, int h, int w, int pitch, int r, const TapsT<T>& tt, void* Ix,
                       void* Iy, void* gm, void* orient, cudaStream_t stream)
{
    switch (r) {
#define TOED_DIRECT_CASE(RR) \
    case RR: return launch_direct<T, RR>(pixels, dtype, h, w, pitch, tt, Ix, Iy, gm, orient, stream);
    TOED_DIRECT_CASE(1) TOED_DIRECT_CASE(2) TOED_DIRECT_CASE(3) TOED_DIRECT_CASE(4)
    TOED_DIRECT_CASE(5) TOED_DIRECT_CASE(6) TOED_DIRECT_CASE(7) TOED_DIRECT_CASE(8)
    TOED_DIRECT_CASE(9) TOED_DIRECT_CASE(10) TOED_DIRECT_CASE(11) TOED_DIRECT_CASE(12)
#undef TOED_DIRECT_CASE
    default: return cudaErrorInvalidValue;
    }
}

// Taps for the planes kernels: the library's FP32 taps for float planes,
// the formula in FP64 for double planes, or the caller's table.
template <typename T>
void planes_taps(float sigma, int r, const double* taps, TapsT<T>& tt)
{
    TapBlock tb;
    make_taps((double)sigma, r, &tb);
    std::memset(&tt, 0, sizeof(tt));
    // FP64 planes take the taps straight from the formula in double
    const double nrm = std::sqrt(2.0 * 3.14159265358979323846);
    for (int sh = 0; sh < 2; ++sh)
        for (int k = 0; k < 2 * r + 3; ++k) {
            const double x = (double)(k - (r + 1)) + (sh ? 0.5 : 0.0), s = sigma;
            const double e = std::exp(-(x * x) / (2.0 * s * s));
            const double vals[4] = {e / (nrm * s), (-x * e) / (nrm * s * s * s),
                                    ((x * x - s * s) * e) / (nrm * s * s * s * s * s),
                                    ((x * (3.0 * s * s - x * x)) * e) / (nrm * s * s * s * s * s * s * s)};
            for (int f = 0; f < 4; ++f) tt.v[4 * sh + f][k] = sizeof(T) == 4 ? (T)tb.v[4 * sh + f][k] : (T)vals[f];
        }
    if (taps)
        for (int f = 0; f < 8; ++f)
            for (int k = 0; k < 2 * r + 3; ++k) tt.v[f][k] = (T)taps[f * (2 * r + 3) + k];
}

template <typename T>
cudaError_t run_planes(const void* pixels, int dtype, int h, int w, int pitch, float sigma, int r,
                       const double* taps, void* Ix, void* Iy, void* gm, void* orient, cudaStream_t stream)
{
    TapsT<T> tt;
    planes_taps<T>(sigma, r, taps, tt);
    const int NR = TH + 2 * r + 2, NIN = TW + 2 * r + 2;
    const size_t smem = sizeof(T) * ((size_t)NR * NIN + 12 * (size_t)NR * TW);
    cudaError_t e = cudaFuncSetAttribute((const void*)planes_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((w + TW - 1) / TW, (h + TH - 1) / TH);
    planes_kernel<T><<<grid, 256, smem, stream>>>(pixels, dtype, h, w, (long long)pitch, r, tt, (T*)Ix, (T*)Iy,
                                                  (T*)gm, (T*)orient);
    return cudaGetLastError();
}

}  // namespace
}  // namespace toed

using namespace toed;

extern "C" toed_status toed_convolve_planes(const void* pixels, int dtype, int h, int w, int pitch, float sigma,
                                            int radius, const double* taps, int planes_dtype, void* Ix, void* Iy,
                                            void* grad_mag, void* orient, cudaStream_t stream)
{
    if (!pixels || !Ix || !Iy || !grad_mag || !orient || h <= 0 || w <= 0 || pitch < w) return TOED_ERR_INVALID_ARG;
    if (!(sigma > 0.f) && !taps) return TOED_ERR_INVALID_ARG;
    if (taps && radius <= 0) return TOED_ERR_INVALID_ARG;
    if (dtype != TOED_U8 && dtype != TOED_F32 && dtype != TOED_F64) return TOED_ERR_UNSUPPORTED;
    const int r = radius > 0 ? radius : (int)std::ceil(4.0 * (double)sigma);
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    cudaError_t e;
    if (planes_dtype == TOED_F32)
        e = run_planes<float>(pixels, dtype, h, w, pitch, sigma, r, taps, Ix, Iy, grad_mag, orient, stream);
    else if (planes_dtype == TOED_F64)
        e = run_planes<double>(pixels, dtype, h, w, pitch, sigma, r, taps, Ix, Iy, grad_mag, orient, stream);
    else
        return TOED_ERR_INVALID_ARG;
    return e == cudaSuccess ? TOED_OK : TOED_ERR_CUDA;
}

extern "C" toed_status toed_convolve_planes_direct(const void* pixels, int dtype, int h, int w, int pitch,
                                                   float sigma, int radius, const double* taps, int planes_dtype,
                                                   void* Ix, void* Iy, void* grad_mag, void* orient,
                                                   cudaStream_t stream)
{
    if (!pixels || !Ix || !Iy || !grad_mag || !orient || h <= 0 || w <= 0 || pitch < w) return TOED_ERR_INVALID_ARG;
    if (!(sigma > 0.f) && !taps) return TOED_ERR_INVALID_ARG;
    if (taps && radius <= 0) return TOED_ERR_INVALID_ARG;
    if (dtype != TOED_U8 && dtype != TOED_F32 && dtype != TOED_F64) return TOED_ERR_UNSUPPORTED;
    const int r = radius > 0 ? radius : (int)std::ceil(4.0 * (double)sigma);
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    cudaError_t e;
    if (planes_dtype == TOED_F32) {
        TapsT<float> tt;
        planes_taps<float>(sigma, r, taps, tt);
        e = run_direct<float>(pixels, dtype, h, w, pitch, r, tt, Ix, Iy, grad_mag, orient, stream);
    } else if (planes_dtype == TOED_F64) {
        TapsT<double> tt;
        planes_taps<double>(sigma, r, taps, tt);
        e = run_direct<double>(pixels, dtype, h, w, pitch, r, tt, Ix, Iy, grad_mag, orient, stream);
    } else {
        return TOED_ERR_INVALID_ARG;
    }
    return e == cudaSuccess ? TOED_OK : TOED_ERR_CUDA;
}

extern "C" toed_status toed_nms_planes(int planes_dtype, int interp_h, int interp_w, const void* Ix, const void* Iy,
                                       const void* grad_mag, float threshold, int border, void* pos_x_map,
                                       void* pos_y_map, cudaStream_t stream)
{
    if (!Ix || !Iy || !grad_mag || !pos_x_map || !pos_y_map || interp_h <= 0 || interp_w <= 0 || border < 1)
        return TOED_ERR_INVALID_ARG;
    const long long n = (long long)interp_h * interp_w;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
    if (planes_dtype == TOED_F32)
        nms_kernel<float><<<blocks, 256, 0, stream>>>(interp_h, interp_w, (const float*)Ix, (const float*)Iy,
                                                      (const float*)grad_mag, threshold, border, (float*)pos_x_map,
                                                      (float*)pos_y_map);
    else if (planes_dtype == TOED_F64)
        nms_kernel<double><<<blocks, 256, 0, stream>>>(interp_h, interp_w, (const double*)Ix, (const double*)Iy,
                                                       (const double*)grad_mag, (double)threshold, border,
                                                       (double*)pos_x_map, (double*)pos_y_map);
    else
        return TOED_ERR_INVALID_ARG;
    return cudaGetLastError() == cudaSuccess ? TOED_OK : TOED_ERR_CUDA;
}
