// toed_subpix.cu -- subpixel third-order correction of dense edge maps on
// GB300: the reference's SubpixelTOCorrectionCPU<T>::estimate_orientation()
// + run() (subpix_TO_correction/subpix_to_correction.cpp:307-736) as five
// short kernels over a batch of maps.  At interp_n > 0 the maps are first
// bilinearly resized onto the 2^n work grid (tc_resize, :69-90) and the
// kernels below run on that grid; positions come out in original pixels.
//
//
//   tc_orient_nms   one CTA per 32x32 tile: triangle smoothing (r = 4,
//                   symmetric padding), gradient2 with one-sided borders and
//                   the Hessian orientation (:307-375) -- or the caller's
//                   orientation -- then dir = (cos, sin) (:296-305) and NMS
//                   along dir on E with the parabola fit (:413-519); edgels are
//                   compacted in row-major order into staging with a
//                   (row, tile column) segment table and a per-pixel id map.
//   tc_correct      one CTA per tile that holds edgels: the eight circular
//                   separable Gaussian-derivative convolutions (:377-411,
//                   :641-648) fused over the tile + halo in shared memory
//                   (6 row filters, 8 column filters), then per edgel the Keys
//                   bicubic samples of ten planes (:521-556) and the corrected
//                   orientation (:663-694).
//   tc_isolate      per segment: an edgel survives if another lies within
//                   the neighbour radius in the reference's 3x3 cell grid
//                   (:563-621), found through the id map.
//   tc_compact      per segment: stable in-place compaction of survivors.
//   then the ordering pass of toed_finalize.cu, and tc_dense (two passes)
//   for the dense TO_E / TO_O maps at round(x, y), later edgels winning
//   (:708-715).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

constexpr int kT = 32;   // tile side (pixels)
constexpr int kTriR = 4; // triangle filter radius (:316)

struct SubMap {
    const void* E;       // the map the kernels read: the caller's, or its work-grid resize
    const void* theta;
    long long pitch;
    long long px_base;   // offset of this map in the per-pixel scratch planes
    void* TO_E;
    void* TO_O;
    int h, w, dtype;     // work grid (the original grid at interp_n = 0)
    int oh, ow;          // original grid (dense TO maps)
    int scale, margin;   // 2^interp_n; NMS margin 3 * 2^interp_n (:628-630)
    int ntx, nty;
    int tile_base;       // first spatial tile of this map
    long long seg_base;  // first (row, tile column) segment, kSegTile aligned
    int seg_tile_base;   // first segment tile
};

struct SubParams {
    float g[3][kMaxTaps];  // G, dG, d2G at integer offsets -r..r (index k <-> k - r)
    int r;
    float thresh;
    double nbr;
    int hyb;
    int out_f64;
    int n_maps;
    int n_tiles;
    Scratch sc;
    float2* dir;         // per pixel (cos, sin) of the NMS direction
    int* eid;            // per pixel staging index of its edgel or -1
    int* img_count;      // per map number of NMS edgels (before removal)
    int* win;            // per pixel winning list index for the dense maps
    unsigned char* keep; // per staged edgel: survives the isolation test
    int n_seg_tiles;
    SubMap m[kBatchMax];
};

__device__ __forceinline__ int wrap_sym(int i, int n)
{  // :47-55
    if (n <= 1) return 0;
    while (i < 0 || i >= n) i = (i < 0) ? -i - 1 : 2 * n - i - 1;
    return i;
}

__device__ __forceinline__ int wrap_circ(int i, int n)
{  // :40-45
    int r = i % n;
    return r < 0 ? r + n : r;
}

__device__ __forceinline__ float load_map(const void* p, int dtype, long long o)
{
    return dtype == TOED_F64 ? (float)__ldg((const double*)p + o) : __ldg((const float*)p + o);
}

// ---------------------------------------------------------------------------
// Double-float arithmetic (an unevaluated sum hi + lo of two floats, about
// 48 significant bits; Dekker / Knuth error-free transformations with the
// FMA for products).  The Hessian orientation estimate of the HYBRID mode
// runs in it: its second differences of the smoothed map cancel, and in
// plain FP32 the estimated angle at an NMS pixel -- which steers the NMS and
// hence the subpixel position and the corrected orientation -- is off by up
// to 1e-4 rad (and its sign of Oxy can flip), at ~1/50 of the FP64 cost.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return make_float2(s, e);
}
__device__ __forceinline__ float2 df_fast_two_sum(float a, float b)  // |a| >= |b| or a == 0
{
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    const float2 s = df_two_sum(a.x, b.x);
    return df_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
    const float p = __fmul_rn(a.x, b.x);
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, fmaf(a.y, b.x, e));
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 df_mul_f(float a, float2 b)  // a float times a double-float
{
    const float p = __fmul_rn(a, b.x);
    const float e = fmaf(a, b.y, fmaf(a, b.x, -p));
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ float2 df_half(float2 a) { return make_float2(0.5f * a.x, 0.5f * a.y); }  // exact

// The NMS max test's near ties (cp or cm == 2) decided in FP64 on the same
// FP32 inputs, the products exact: f ga against Map (ga - gb) + Mdp gb and
// Mam (ga - gb) + Mdm gb (a few pixels per map; out of line, so that the
// conversions stay off the per-pixel path).
static __device__ __noinline__ void max_test_fp64(float f, float ga, float gb, float Map, float Mdp, float Mam,
                                                  float Mdm, int* cp, int* cm)
{
    const double gad = ga, gbd = gb, d = gad - gbd, fD = (double)f * gad;
    if (*cp == 2) {
        const double fpD = fma((double)Map, d, (double)Mdp * gbd);
        *cp = fD > fpD ? 1 : (fD < fpD ? -1 : 0);
    }
    if (*cm == 2) {
        const double fmD = fma((double)Mam, d, (double)Mdm * gbd);
        *cm = fD > fmD ? 1 : (fD < fmD ? -1 : 0);
    }
}

// a b + c d + e f + g h in FP32 with the products split exactly (FMA) and
// the sum compensated -- the Dot2 algorithm of Ogita, Rump and Oishi
// ("Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005): the
// result is as accurate as if computed in twice the working precision and
// then rounded, which is what the four cancelling products need.
// (The _rn intrinsics keep the compiler from contracting the error terms.)
__device__ __forceinline__ float dot4_comp(float a, float b, float c, float d, float e, float f, float g, float h)
{
    float p = __fmul_rn(a, b), err = fmaf(a, b, -p);
    const float x[3] = {c, e, g}, y[3] = {d, f, h};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float q = __fmul_rn(x[k], y[k]), qe = fmaf(x[k], y[k], -q);
        const float2 t = df_two_sum(p, q);  // p + q = t.x + t.y exactly
        err = __fadd_rn(err, __fadd_rn(t.y, qe));
        p = t.x;
    }
    return __fadd_rn(p, err);
}

// The triangle filter (:316-321), weight (5 - |k|) / 25, as double-floats.
template <int K>
struct TriDF {
    static constexpr double w = (double)(5 - (K < 0 ? -K : K)) / 25.0;
    static constexpr float hi = (float)w;
    static constexpr float lo = (float)(w - (double)hi);
};
__device__ __forceinline__ float2 tri_df(int k)
{
    switch (k) {
    case -4: return make_float2(TriDF<-4>::hi, TriDF<-4>::lo);
    case -3: return make_float2(TriDF<-3>::hi, TriDF<-3>::lo);
    case -2: return make_float2(TriDF<-2>::hi, TriDF<-2>::lo);
    case -1: return make_float2(TriDF<-1>::hi, TriDF<-1>::lo);
    case 0: return make_float2(TriDF<0>::hi, TriDF<0>::lo);
    case 1: return make_float2(TriDF<1>::hi, TriDF<1>::lo);
    case 2: return make_float2(TriDF<2>::hi, TriDF<2>::lo);
    case 3: return make_float2(TriDF<3>::hi, TriDF<3>::lo);
    default: return make_float2(TriDF<4>::hi, TriDF<4>::lo);
    }
}

__device__ __forceinline__ double cubic_w(double s)
{  // Keys kernel, a = -0.5 (:57-67)
    const double a = -0.5;
    const double x = fabs(s);
    if (x <= 1.0) return ((a + 2) * x - (a + 3)) * x * x + 1;
    if (x < 2.0) return ((a * x - 5 * a) * x + 8 * a) * x - 4 * a;
    return 0.0;
}

__device__ __forceinline__ float cubic_wf(float s)
{  // the same kernel in FP32, for interpolation weights of FP32 data
    const float a = -0.5f;
    const float x = fabsf(s);
    if (x <= 1.f) return ((a + 2.f) * x - (a + 3.f)) * x * x + 1.f;
    if (x < 2.f) return ((a * x - 5.f * a) * x + 8.f * a) * x - 4.f * a;
    return 0.f;
}

// ---------------------------------------------------------------------------
// Orientation + NMS
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 5) tc_orient_nms(const __grid_constant__ SubParams p)
{
    constexpr int HE = 6, NE = kT + 2 * HE;  // E region: rows/cols i0-6 .. i0+37
    __shared__ float sE[NE][NE + 1];
    __shared__ float2 sDir[kT][kT];
    __shared__ int sRowCnt[kT], sRowOff[kT], sCandOff[kT + 1];
    __shared__ unsigned sOk[kT];              // per row: candidates the fit accepted
    // the orientation estimate's stages (triangle rows, smoothed map, gradients), dead once the
    // directions are in, then the NMS candidates: one buffer (five CTAs per SM)
    constexpr size_t kTmpB = sizeof(float) * NE * (kT + 4), kSmB = sizeof(float) * (kT + 4) * (kT + 4);
    constexpr size_t kOB = sizeof(float) * (kT + 2) * (kT + 3);
    constexpr size_t kCandB = sizeof(short) * kT * kT, kResB = sizeof(float3) * kT * kT;
    // HYBRID: the triangle rows and the smoothed map as double-floats (no gradient planes)
    constexpr size_t kStageF = kTmpB + kSmB + 2 * kOB, kStageD = 2 * (kTmpB + kSmB);
    constexpr size_t kStageB = kStageF > kStageD ? kStageF : kStageD;
    static_assert(kCandB + kResB <= kStageB, "candidates fit the orientation stages");
    __shared__ __align__(16) unsigned char sStage[kStageB];
    float(*sTmp)[kT + 4] = reinterpret_cast<float(*)[kT + 4]>(sStage);               // cols j0-2 .. j0+33
    float(*sSm)[kT + 4] = reinterpret_cast<float(*)[kT + 4]>(sStage + kTmpB);        // rows/cols -2 .. +33
    float(*sOx)[kT + 3] = reinterpret_cast<float(*)[kT + 3]>(sStage + kTmpB + kSmB);  // -1 .. +32
    float(*sOy)[kT + 3] = reinterpret_cast<float(*)[kT + 3]>(sStage + kTmpB + kSmB + kOB);
    short* sCand = reinterpret_cast<short*>(sStage);  // max-test candidates, row-major (tile pixel a * 32 + b)
    float3* sRes = reinterpret_cast<float3*>(sStage + kCandB);  // per candidate: offset (x, y), |max_f|

    const int t = blockIdx.x;
    const int k = find_image(p.n_maps, t, [&](int i) { return p.m[i].tile_base; });
    const SubMap& M = p.m[k];
    const int h = M.h, w = M.w, dtype = M.dtype;
    const int lt = t - M.tile_base;
    const int ty = lt / M.ntx, tx = lt - ty * M.ntx;
    const int i0 = ty * kT, j0 = tx * kT;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

    const bool inside = i0 - HE >= 0 && j0 - HE >= 0 && i0 - HE + NE <= h && j0 - HE + NE <= w;  // no padding
    for (int q = tid; q < NE * NE; q += blockDim.x) {
        const int a = q / NE, b = q - a * NE;
        const int ii = inside ? i0 - HE + a : wrap_sym(i0 - HE + a, h);
        const int jj = inside ? j0 - HE + b : wrap_sym(j0 - HE + b, w);
        sE[a][b] = load_map(M.E, dtype, (long long)ii * M.pitch + jj);
    }
    __syncthreads();

    // HYBRID: tiles holding an NMS candidate (E > thresh inside the margin)
    // estimate the orientation in double-float arithmetic; the others, whose
    // directions only weight the Hx / Hy maps, in FP32
    bool df_tile = false;
    if (M.theta == nullptr && p.hyb) {
        bool any = false;
        for (int q = tid; q < kT * kT; q += blockDim.x) {
            const int a = q >> 5, b = q & 31, i = i0 + a, j = j0 + b;
            any = any || (i >= M.margin + 1 && i < h - M.margin - 2 && j >= M.margin + 1 && j < w - M.margin - 2 &&
                          sE[a + HE][b + HE] > p.thresh);
        }
        df_tile = __syncthreads_or(any);
    }
    if (df_tile) {
        // the orientation estimate in double-float arithmetic (see
        // df_two_sum); the same sums, in the same order, as the FP32 form
        float2(*sTmpD)[kT + 4] = reinterpret_cast<float2(*)[kT + 4]>(sStage);          // cols j0-2 .. j0+33
        float2(*sSmD)[kT + 4] = reinterpret_cast<float2(*)[kT + 4]>(sStage + 2 * kTmpB);  // rows/cols -2 .. +33
        for (int q = tid; q < NE * (kT + 4); q += blockDim.x) {
            const int a = q / (kT + 4), c = q - a * (kT + 4);
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int qq = -kTriR; qq <= kTriR; ++qq)
                acc = df_add(acc, df_mul_f(sE[a][c + 4 - qq], tri_df(qq)));
            sTmpD[a][c] = acc;
        }
        __syncthreads();
        for (int q = tid; q < (kT + 4) * (kT + 4); q += blockDim.x) {
            const int d = q / (kT + 4), c = q - d * (kT + 4);
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int pp = -kTriR; pp <= kTriR; ++pp) acc = df_add(acc, df_mul(sTmpD[d + 4 - pp][c], tri_df(pp)));
            sSmD[d][c] = acc;
        }
        __syncthreads();
        // gradient2 (:346-355) of the smoothed map and of its gradients, at
        // the tile's pixels, one-sided at the image borders
        auto sm = [&](int i, int j) { return sSmD[i - i0 + 2][j - j0 + 2]; };
        auto ox = [&](int i, int j) {
            return (j == 0) ? df_sub(sm(i, 1), sm(i, 0))
                            : (j == w - 1 ? df_sub(sm(i, j), sm(i, j - 1)) : df_half(df_sub(sm(i, j + 1), sm(i, j - 1))));
        };
        auto oy = [&](int i, int j) {
            return (i == 0) ? df_sub(sm(1, j), sm(0, j))
                            : (i == h - 1 ? df_sub(sm(i, j), sm(i - 1, j)) : df_half(df_sub(sm(i + 1, j), sm(i - 1, j))));
        };
        for (int q = tid; q < kT * kT; q += blockDim.x) {
            const int a = q >> 5, b = q & 31;
            const int i = i0 + a, j = j0 + b;
            if (i >= h || j >= w) continue;
            const float2 oxx = (j == 0) ? df_sub(ox(i, 1), ox(i, 0))
                                        : (j == w - 1 ? df_sub(ox(i, j), ox(i, j - 1))
                                                      : df_half(df_sub(ox(i, j + 1), ox(i, j - 1))));
            const float2 oxy = (j == 0) ? df_sub(oy(i, 1), oy(i, 0))
                                        : (j == w - 1 ? df_sub(oy(i, j), oy(i, j - 1))
                                                      : df_half(df_sub(oy(i, j + 1), oy(i, j - 1))));
            const float2 oyy = (i == 0) ? df_sub(oy(1, j), oy(0, j))
                                        : (i == h - 1 ? df_sub(oy(i, j), oy(i - 1, j))
                                                      : df_half(df_sub(oy(i + 1, j), oy(i - 1, j))));
            // the sign of Oxy and x = Oxx + 1e-5 decided on the double-float values
            const float sgn = (oxy.x < 0.f) ? 1.f : ((oxy.x > 0.f) ? -1.f : 0.f);
            constexpr double kEps = 1e-5;
            constexpr float kEpsHi = (float)kEps, kEpsLo = (float)(kEps - (double)kEpsHi);
            const float2 xd = df_add(oxx, make_float2(kEpsHi, kEpsLo));
            const float x = xd.x, y = oyy.x * sgn;
            float2 d;
            if (x != 0.f) {
                // (cos, sin) of atan(y / x) wrapped to [0, pi) (:370-374, :296-305), as below
                const float rn = rsqrtf(fmaf(x, x, y * y));
                const float cx = fabsf(x) * rn, sy = copysignf(1.f, x) * y * rn;
                d = (x * y < 0.f) ? make_float2(-cx, -sy) : make_float2(cx, sy);
            } else {  // atan(y / 0): pi / 2 after the wrap, NaN for 0 / 0 (as the reference)
                float a2 = fmodf(atanf(y / x), 3.14159265358979323846f);
                if (a2 < 0.f) a2 += 3.14159265358979323846f;
                float sn, cs;
                sincosf(a2, &sn, &cs);
                d = make_float2(cs, sn);
            }
            sDir[a][b] = d;
            p.dir[M.px_base + (long long)i * w + j] = d;
        }
        __syncthreads();
    } else if (M.theta == nullptr) {
        const float tri[9] = {1.f / 25, 2.f / 25, 3.f / 25, 4.f / 25, 5.f / 25, 4.f / 25, 3.f / 25, 2.f / 25, 1.f / 25};
        for (int q = tid; q < NE * (kT + 4); q += blockDim.x) {
            const int a = q / (kT + 4), c = q - a * (kT + 4);
            float acc = 0.f;
#pragma unroll
            for (int qq = -kTriR; qq <= kTriR; ++qq) acc += sE[a][c + 4 - qq] * tri[qq + kTriR];
            sTmp[a][c] = acc;
        }
        __syncthreads();
        for (int q = tid; q < (kT + 4) * (kT + 4); q += blockDim.x) {
            const int d = q / (kT + 4), c = q - d * (kT + 4);
            float acc = 0.f;
#pragma unroll
            for (int pp = -kTriR; pp <= kTriR; ++pp) acc += sTmp[d + 4 - pp][c] * tri[pp + kTriR];
            sSm[d][c] = acc;
        }
        __syncthreads();
        // gradient2 (:346-355): central differences, one-sided at the borders
        for (int q = tid; q < (kT + 2) * (kT + 2); q += blockDim.x) {
            const int e = q / (kT + 2), f = q - e * (kT + 2);
            const int i = i0 - 1 + e, j = j0 - 1 + f;
            float ox = 0.f, oy = 0.f;
            if (i >= 0 && i < h && j >= 0 && j < w) {
                const int d = e + 1, c = f + 1;
                ox = (j == 0) ? sSm[d][c + 1] - sSm[d][c]
                              : (j == w - 1 ? sSm[d][c] - sSm[d][c - 1] : 0.5f * (sSm[d][c + 1] - sSm[d][c - 1]));
                oy = (i == 0) ? sSm[d + 1][c] - sSm[d][c]
                              : (i == h - 1 ? sSm[d][c] - sSm[d - 1][c] : 0.5f * (sSm[d + 1][c] - sSm[d - 1][c]));
            }
            sOx[e][f] = ox;
            sOy[e][f] = oy;
        }
        __syncthreads();
    }
    const float PI_F = 3.14159265358979323846f;
    for (int q = tid; q < kT * kT && !df_tile; q += blockDim.x) {
        const int a = q >> 5, b = q & 31;
        const int i = i0 + a, j = j0 + b;
        float th = 0.f;
        if (i < h && j < w) {
            if (M.theta) {
                th = load_map(M.theta, dtype, (long long)i * M.pitch + j);
            } else {
                const int e = a + 1, f = b + 1;
                const float oxx = (j == 0) ? sOx[e][f + 1] - sOx[e][f]
                                           : (j == w - 1 ? sOx[e][f] - sOx[e][f - 1] : 0.5f * (sOx[e][f + 1] - sOx[e][f - 1]));
                const float oxy = (j == 0) ? sOy[e][f + 1] - sOy[e][f]
                                           : (j == w - 1 ? sOy[e][f] - sOy[e][f - 1] : 0.5f * (sOy[e][f + 1] - sOy[e][f - 1]));
                const float oyy = (i == 0) ? sOy[e + 1][f] - sOy[e][f]
                                           : (i == h - 1 ? sOy[e][f] - sOy[e - 1][f] : 0.5f * (sOy[e + 1][f] - sOy[e - 1][f]));
                const float sgn = (oxy < 0.f) ? 1.f : ((oxy > 0.f) ? -1.f : 0.f);
                const float x = oxx + 1e-5f, y = oyy * sgn;
                if (x != 0.f) {
                    // th = atan(y / x) (:370-371) lies in (-pi/2, pi/2), so
                    // wrap_mod_pi (:216-222) adds pi exactly when th < 0, and
                    // compute_dir_from_theta (:296-305) is (cos, sin) of that:
                    // (|x|, y sgn x) / |(x, y)|, negated when x y < 0
                    const float rn = rsqrtf(fmaf(x, x, y * y));
                    const float cx = fabsf(x) * rn, sy = copysignf(1.f, x) * y * rn;
                    const float2 d = (x * y < 0.f) ? make_float2(-cx, -sy) : make_float2(cx, sy);
                    sDir[a][b] = d;
                    p.dir[M.px_base + (long long)i * w + j] = d;
                    continue;
                }
                th = atanf(y / x);
            }
            // wrap_mod_pi (:216-222), then compute_dir_from_theta (:296-305)
            float a2 = fmodf(th, PI_F);
            if (a2 < 0.f) a2 += PI_F;
            float sn, cs;
            sincosf(a2, &sn, &cs);
            sDir[a][b] = make_float2(cs, sn);
            p.dir[M.px_base + (long long)i * w + j] = make_float2(cs, sn);
        }
    }
    __syncthreads();

    // NMS along dir on E (:424-514), margin mg: i, j in [mg + 1, dim - mg - 2).
    // 1. per pixel, the max test along the sector's interpolated neighbours.
    //    HYBRID decides in FP64 without a division: with ga = |g| along the
    //    major axis (> 0) and gb along the minor one, slope = gb / ga, so
    //    f > fp  <=>  f ga > Map (ga - gb) + Mdp gb, whose products of FP32
    //    values are exact or rounded once in FP64.
    unsigned bal1[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int a = wid + 8 * u, b = lane;
        const int i = i0 + a, j = j0 + b;
        bool cand = false;
        if (i >= M.margin + 1 && i < h - M.margin - 2 && j >= M.margin + 1 && j < w - M.margin - 2) {
            const float f = sE[a + HE][b + HE];
            const float2 g = sDir[a][b];
            if (f > p.thresh && !(fabsf(g.x) < 1e-5f && fabsf(g.y) < 1e-5f)) {
                // eight sectors of :453-493 in closed form (x-major when |gx| >= |gy|)
                const bool xmaj = fabsf(g.x) >= fabsf(g.y);
                const int sx = g.x >= 0.f ? 1 : -1, sy = g.y >= 0.f ? 1 : -1;
                const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
                const float Map = sE[a + HE + ar][b + HE + ac], Mdp = sE[a + HE + sy][b + HE + sx];
                const float Mam = sE[a + HE - ar][b + HE - ac], Mdm = sE[a + HE - sy][b + HE - sx];
                if (p.hyb) {
                    // FP32 first; the FP64 form only where f lies within the FP32
                    // rounding bound of fp or fm (a few pixels per map)
                    const float ga = xmaj ? fabsf(g.x) : fabsf(g.y), gb = xmaj ? fabsf(g.y) : fabsf(g.x);
                    const float fpS = fmaf(Map, ga - gb, Mdp * gb), fmS = fmaf(Mam, ga - gb, Mdm * gb);
                    const float fS = f * ga;
                    // |FP32 - exact| <= ~3e-7 (|f| + |Map| + |Mdp| + |Mam| + |Mdm|) ga; 30x margin.
                    // Neighbours equal to f (a plateau, e.g. a clipped ridge) tie
                    // exactly in the FP64 form too: decided without it.
                    const float tol = 1e-5f * ga * (fabsf(f) + fabsf(Map) + fabsf(Mdp) + fabsf(Mam) + fabsf(Mdm));
                    int cp = (Map == f && Mdp == f) ? 0 : (fS - fpS > tol ? 1 : (fpS - fS > tol ? -1 : 2));
                    int cm = (Mam == f && Mdm == f) ? 0 : (fS - fmS > tol ? 1 : (fmS - fS > tol ? -1 : 2));
                    if (cp == 2 || cm == 2) max_test_fp64(f, ga, gb, Map, Mdp, Mam, Mdm, &cp, &cm);
                    cand = (cm > 0 && cp >= 0) || (cm >= 0 && cp > 0);  // :466-468
                } else {
                    const float md = sqrtf(g.x * g.x + g.y * g.y);
                    const float nx = g.x / md, ny = g.y / md;
                    const float sl = xmaj ? fabsf(ny) / fabsf(nx) : fabsf(nx) / fabsf(ny);
                    const float fp = Map * (1 - sl) + Mdp * sl, fm = Mam * (1 - sl) + Mdm * sl;
                    cand = (f > fm && f >= fp) || (f >= fm && f > fp);
                }
            }
        }
        bal1[u] = __ballot_sync(0xffffffffu, cand);
        if (lane == 0) sRowCnt[a] = __popc(bal1[u]);
    }
    if (tid < kT) sOk[tid] = 0u;
    __syncthreads();
    if (wid == 0) {
        const int cnt = sRowCnt[lane];
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        sCandOff[lane] = incl - cnt;
        if (lane == 31) sCandOff[kT] = incl;
    }
    __syncthreads();
    const unsigned ltm = (1u << lane) - 1u;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int a = wid + 8 * u;
        if ((bal1[u] >> lane) & 1u) sCand[sCandOff[a] + __popc(bal1[u] & ltm)] = (short)(a * kT + lane);
    }
    __syncthreads();
    // 2. the parabola fit of the candidates, a thread each (:466-512): FP64
    //    in HYBRID; subpixel offsets and |max_f| kept per candidate slot
    const int ncand = sCandOff[kT];
    for (int c = tid; c < ncand; c += blockDim.x) {
        const int a = sCand[c] / kT, b = sCand[c] - (sCand[c] / kT) * kT;
        const float f = sE[a + HE][b + HE];
        const float2 g = sDir[a][b];
        const bool xmaj = fabsf(g.x) >= fabsf(g.y);
        const int sx = g.x >= 0.f ? 1 : -1, sy = g.y >= 0.f ? 1 : -1;
        const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
        const float Map = sE[a + HE + ar][b + HE + ac], Mdp = sE[a + HE + sy][b + HE + sx];
        const float Mam = sE[a + HE - ar][b + HE - ac], Mdm = sE[a + HE - sy][b + HE - sx];
        bool ok = false;
        float dx = 0.f, dy = 0.f, mag = 0.f;
        if (p.hyb) {
            // fp - fm and fm + fp - 2f cancel.  With fp = Map + s (Mdp - Map) and
            // fm = Mam + s (Mdm - Mam) both come from differences of nearly equal
            // FP32 values (exact within a factor 2 of each other), the weight
            // applied last -- no full-scale sum is rounded before the
            // cancellation; the well-conditioned rest in FP32.  s* = -B / (2A)
            // with A = (fm + fp - 2f) / (2 s^2), B = (fp - fm) / (2 s) (:496-505)
            const float md = sqrtf(g.x * g.x + g.y * g.y);
            const float nx = g.x / md, ny = g.y / md;
            const float sl = xmaj ? fabsf(ny) / fabsf(nx) : fabsf(nx) / fabsf(ny);
            const float dA = Map - Mam, dD = Mdp - Mdm;
            const float eA = (Map - f) + (Mam - f), eD = (Mdp - f) + (Mdm - f);
            const float num = fmaf(sl, dD - dA, dA), den = fmaf(sl, eD - eA, eA);
            const float s = sqrtf(1.f + sl * sl);
            if (!(fabsf(den) < 2e-16f * (s * s))) {  // |A| < 1e-16 (:502)
                const float ss = -0.5f * num * s / den;
                const float mf = f - 0.125f * num * num / den;  // A s*^2 + B s* + f
                if (fabsf(ss) <= 1.41421356f) {
                    ok = true;
                    dx = ss * nx;
                    dy = ss * ny;
                    mag = fabsf(mf);
                }
            }
        } else {
            const float md = sqrtf(g.x * g.x + g.y * g.y);
            const float nx = g.x / md, ny = g.y / md;
            const float sl = xmaj ? fabsf(ny) / fabsf(nx) : fabsf(nx) / fabsf(ny);
            const float fp = Map * (1 - sl) + Mdp * sl, fm = Mam * (1 - sl) + Mdm * sl;
            const float s = sqrtf(1 + sl * sl);
            const float A = (fm + fp - 2 * f) / (2 * s * s), B = (fp - fm) / (2 * s);
            if (!(fabsf(A) < 1e-16f)) {
                const float ss = -B / (2 * A);
                const float mf = A * ss * ss + B * ss + f;
                if (fabsf(ss) <= 1.41421356f) {
                    ok = true;
                    dx = ss * nx;
                    dy = ss * ny;
                    mag = fabsf(mf);
                }
            }
        }
        sRes[c] = make_float3(dx, dy, mag);
        if (ok) atomicOr(&sOk[a], 1u << b);
    }
    __syncthreads();
    // 3. the edgels in row-major order: staging slots, segment table, id map
    if (wid == 0) {
        const int cnt = __popc(sOk[lane]);
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int base = 0;
        if (lane == 0 && total > 0) {
            base = atomicAdd(&p.sc.words[1], total);
            atomicAdd(&p.img_count[k], total);
            if ((long long)base + total > p.sc.staging_cap) atomicOr(&p.sc.words[2], TOED_FLAG_STAGING_FULL);
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        sRowOff[lane] = base + incl - cnt;
        // segment (row, tile column) -> {staging offset, count}
        const int i = i0 + lane;
        if (i < h) p.sc.seg[M.seg_base + (long long)i * M.ntx + tx] = make_int2(base + incl - cnt, cnt);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int a = wid + 8 * u, b = lane;
        const int i = i0 + a, j = j0 + b;
        if (i >= h || j >= w) continue;
        const unsigned okm = sOk[a];
        int id = -1;
        if ((okm >> lane) & 1u) {
            id = sRowOff[a] + __popc(okm & ltm);
            if (id < p.sc.staging_cap) {
                // positions and strength packed as (pixel, FP32 offset) / FP32 bits:
                // tc_correct, a thread per edgel, forms the doubles (no FP64
                // instruction here, where every warp-row with an edgel would pay it)
                const float3 r = sRes[sCandOff[a] + __popc(bal1[u] & ltm)];
                p.sc.staging[id] = make_double4_32a(__hiloint2double(j, __float_as_int(r.x)),
                                                    __hiloint2double(i, __float_as_int(r.y)), 0.0,
                                                    __hiloint2double(0, __float_as_int(r.z)));
                p.sc.staging_idx[id] = i * w + j;
            } else {
                id = -1;
            }
        }
        p.eid[M.px_base + (long long)i * w + j] = id;
    }
}

// ---------------------------------------------------------------------------
// Fused convolutions + per-edgel orientation correction
// ---------------------------------------------------------------------------
template <int R>
struct CorrCfg {
    static constexpr int HB = 3;                  // bicubic reach around a tile pixel
    static constexpr int NO = kT + 2 * HB;        // 38: conv output region side
    static constexpr int NI = NO + 2 * R;         // input region side
    // Hx, Hy live through the whole kernel; E only until the row pass, after
    // which its space (grown to 5 planes) takes the column planes Px Py Pxx
    // Pxy Pyy; the row-pass planes 0-2 are dead once those are done and take
    // Hxx Hyy Hxy.  About 101 KB at r = 8: two CTAs per SM.
    static constexpr int NA = (NI * NI > 5 * NO * NO) ? NI * NI : 5 * NO * NO;
    static constexpr size_t off_Hx = 0;                                     // [NI][NI]
    static constexpr size_t off_Hy = off_Hx + sizeof(float) * NI * NI;      // [NI][NI]
    static constexpr size_t off_E = off_Hy + sizeof(float) * NI * NI;       // [NI][NI], then 5 x [NO][NO]
    static constexpr size_t off_row = off_E + sizeof(float) * NA;           // 6 x [NI][NO], then 3 x [NO][NO]
    static constexpr size_t off_colA = off_E;
    static constexpr size_t off_colB = off_row;
    static_assert(3 * NO * NO <= 3 * NI * NO, "Hxx Hyy Hxy fit in the dead row planes 0-2");
    static constexpr size_t off_misc = off_row + sizeof(float) * 6 * NI * NO;
    static constexpr size_t smem = off_misc + sizeof(int) * 2 * (kT + 1);
};

template <int R>
__global__ void __launch_bounds__(512, 2) tc_correct(const __grid_constant__ SubParams p)
{
    using C = CorrCfg<R>;
    constexpr int NI = C::NI, NO = C::NO, HB = C::HB;
    extern __shared__ __align__(16) unsigned char smem[];
    float* sE = reinterpret_cast<float*>(smem + C::off_E);
    float* sHx = reinterpret_cast<float*>(smem + C::off_Hx);
    float* sHy = reinterpret_cast<float*>(smem + C::off_Hy);
    float* sRow = reinterpret_cast<float*>(smem + C::off_row);
    float* sColA = reinterpret_cast<float*>(smem + C::off_colA);  // Px Py Pxx Pxy Pyy
    float* sColB = reinterpret_cast<float*>(smem + C::off_colB);  // Hxx Hyy Hxy
    int* sOff = reinterpret_cast<int*>(smem + C::off_misc);  // [kT+1] exclusive prefix of row counts
    int* sSegOff = sOff + kT + 1;                             // [kT] staging offsets

    const int t = blockIdx.x;
    const int k = find_image(p.n_maps, t, [&](int i) { return p.m[i].tile_base; });
    const SubMap& M = p.m[k];
    const int h = M.h, w = M.w;
    const int lt = t - M.tile_base;
    const int ty = lt / M.ntx, tx = lt - ty * M.ntx;
    const int i0 = ty * kT, j0 = tx * kT;
    const int tid = threadIdx.x;

    if (tid < 32) {
        const int i = i0 + tid;
        int2 sg = make_int2(0, 0);
        if (i < h) sg = p.sc.seg[M.seg_base + (long long)i * M.ntx + tx];
        int incl = sg.y;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (tid >= d) incl += y;
        }
        sOff[tid + 1] = incl;
        if (tid == 0) sOff[0] = 0;
        sSegOff[tid] = sg.x;
    }
    __syncthreads();
    const int n_edg = sOff[kT];
    if (n_edg == 0) return;  // tiles without edgels need no convolution

    // inputs with circular wrap: E, Hx = E dirx, Hy = E diry (:634-638)
    const int ri = i0 - HB - R, rj = j0 - HB - R;
    const bool inside = ri >= 0 && rj >= 0 && ri + NI <= h && rj + NI <= w;  // no wrap needed
    for (int q = tid; q < NI * NI; q += blockDim.x) {
        const int a = q / NI, b = q - a * NI;
        const int ii = inside ? ri + a : wrap_circ(ri + a, h), jj = inside ? rj + b : wrap_circ(rj + b, w);
        const float e = load_map(M.E, M.dtype, (long long)ii * M.pitch + jj);
        const float2 d = p.dir[M.px_base + (long long)ii * w + jj];
        sE[q] = e;
        sHx[q] = e * d.x;
        sHy[q] = e * d.y;
    }
    __syncthreads();
    // row pass (along j): E -> G, dG, d2G ; Hx -> dG ; Hy -> G, dG
    // out(x) = sum_q src(x - q) k(q)  (:392-396).  A thread takes 4
    // consecutive outputs of a row and slides one window of 2r + 4 inputs.
    constexpr int G = 4, NG = (NO + G - 1) / G, NW = 2 * R + G;
    for (int q = tid; q < NI * NG; q += blockDim.x) {
        const int a = q / NG, c0 = (q - a * NG) * G;
        float acc[6][G];
#pragma unroll
        for (int f = 0; f < 6; ++f)
#pragma unroll
            for (int o = 0; o < G; ++o) acc[f][o] = 0.f;
#pragma unroll
        for (int src = 0; src < 3; ++src) {
            const float* row = (src == 0 ? sE : (src == 1 ? sHx : sHy)) + a * NI + c0;
            float win[NW];
#pragma unroll
            for (int t = 0; t < NW; ++t) win[t] = (c0 + t < NI) ? row[t] : 0.f;
#pragma unroll
            for (int qq = -R; qq <= R; ++qq) {
                const float g0 = p.g[0][qq + R], g1 = p.g[1][qq + R], g2 = p.g[2][qq + R];
#pragma unroll
                for (int o = 0; o < G; ++o) {
                    const float x = win[o + R - qq];  // src(c0 + o - qq), window index o + R - qq
                    if (src == 0) {
                        acc[0][o] = fmaf(x, g0, acc[0][o]);
                        acc[1][o] = fmaf(x, g1, acc[1][o]);
                        acc[2][o] = fmaf(x, g2, acc[2][o]);
                    } else if (src == 1) {
                        acc[3][o] = fmaf(x, g1, acc[3][o]);
                    } else {
                        acc[4][o] = fmaf(x, g0, acc[4][o]);
                        acc[5][o] = fmaf(x, g1, acc[5][o]);
                    }
                }
            }
        }
#pragma unroll
        for (int o = 0; o < G; ++o)
            if (c0 + o < NO)
#pragma unroll
                for (int f = 0; f < 6; ++f) sRow[(f * NI + a) * NO + c0 + o] = acc[f][o];
    }
    __syncthreads();
    // column pass (along i) (:641-648): first Px Py Pxx Pxy Pyy from the E
    // row planes 0-2, then Hxx Hyy Hxy from planes 3-5 into the space of
    // planes 0-2; a thread takes 4 consecutive output rows of a column
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        for (int q = tid; q < NG * NO; q += blockDim.x) {
            const int a0 = (q / NO) * G, c = q - (q / NO) * NO;
            float o0[G], o1[G], o2[G], o3[G], o4[G];
#pragma unroll
            for (int o = 0; o < G; ++o) o0[o] = o1[o] = o2[o] = o3[o] = o4[o] = 0.f;
#pragma unroll
            for (int f = 3 * half; f < 3 * half + 3; ++f) {
                // rows a0 .. a0 + 2r + 3 of row-pass plane f at column c (output row a uses row a + R - pp)
                const float* col = sRow + (f * NI + a0) * NO + c;
                float win[NW];
#pragma unroll
                for (int t = 0; t < NW; ++t) win[t] = (a0 + t < NI) ? col[t * NO] : 0.f;
#pragma unroll
                for (int pp = -R; pp <= R; ++pp) {
                    const float g0 = p.g[0][pp + R], g1 = p.g[1][pp + R], g2 = p.g[2][pp + R];
#pragma unroll
                    for (int o = 0; o < G; ++o) {
                        const float x = win[o + R - pp];
                        if (f == 0) {          // eG
                            o1[o] = fmaf(x, g1, o1[o]);  // Py  (G, dG)  E
                            o4[o] = fmaf(x, g2, o4[o]);  // Pyy (G, d2G) E
                        } else if (f == 1) {   // edG
                            o0[o] = fmaf(x, g0, o0[o]);  // Px  (dG, G)  E
                            o3[o] = fmaf(x, g1, o3[o]);  // Pxy (dG, dG) E
                        } else if (f == 2) {   // ed2G
                            o2[o] = fmaf(x, g0, o2[o]);  // Pxx (d2G, G) E
                        } else if (f == 3) {   // xdG
                            o0[o] = fmaf(x, g0, o0[o]);  // Hxx (dG, G)  Hx
                        } else if (f == 4) {   // yG
                            o1[o] = fmaf(x, g1, o1[o]);  // Hyy (G, dG)  Hy
                        } else {               // ydG
                            o2[o] = fmaf(x, g0, o2[o]);  // Hxy (dG, G)  Hy
                        }
                    }
                }
            }
#pragma unroll
            for (int o = 0; o < G; ++o) {
                if (a0 + o >= NO) break;
                const int qo = (a0 + o) * NO + c;
                if (half == 0) {
                    sColA[0 * NO * NO + qo] = o0[o];
                    sColA[1 * NO * NO + qo] = o1[o];
                    sColA[2 * NO * NO + qo] = o2[o];
                    sColA[3 * NO * NO + qo] = o3[o];
                    sColA[4 * NO * NO + qo] = o4[o];
                } else {
                    sColB[0 * NO * NO + qo] = o0[o];
                    sColB[1 * NO * NO + qo] = o1[o];
                    sColB[2 * NO * NO + qo] = o2[o];
                }
            }
        }
        __syncthreads();
    }
    // per edgel: Keys bicubic of ten planes at (sx, sy), clamp to the image
    // (:521-556).  The interpolation is a short weighted sum of FP32
    // convolution outputs and runs in FP32; the F vector, whose four products
    // can cancel, is a compensated dot product of the interpolated values
    // (HYBRID, dot4_comp).
    const double inv_scale = 1.0 / (double)M.scale;  // 2^-interp_n: the products below are exact
    for (int e = tid; e < n_edg; e += blockDim.x) {
        int row = 0;  // last row with sOff[row] <= e
#pragma unroll
        for (int st = 16; st >= 1; st >>= 1)
            if (row + st < kT && sOff[row + st] <= e) row += st;
        const long long sidx = (long long)sSegOff[row] + (e - sOff[row]);
        if (sidx >= p.sc.staging_cap) continue;
        double4_32a rec = p.sc.staging[sidx];
        // unpack tc_orient_nms's (pixel, FP32 offset) positions and FP32 strength
        const int cj = __double2hiint(rec.x), ci = __double2hiint(rec.y);
        const float ox = __int_as_float(__double2loint(rec.x)), oy = __int_as_float(__double2loint(rec.y));
        const double sx = p.hyb ? (double)cj + (double)ox : (double)((float)cj + ox);
        const double sy = p.hyb ? (double)ci + (double)oy : (double)((float)ci + oy);
        rec.w = (double)__int_as_float(__double2loint(rec.w));
        // cell and fraction of the position: from the pixel and its FP32 offset
        // (the fraction correctly rounded to FP32, as (float)(sx - floor(sx)))
        int x0, y0;
        float tfx, tfy;
        if (p.hyb) {
            const float flx = floorf(ox), fly = floorf(oy);
            x0 = cj + (int)flx;
            y0 = ci + (int)fly;
            tfx = ox - flx;
            tfy = oy - fly;
        } else {
            x0 = (int)floor(sx);
            y0 = (int)floor(sy);
            tfx = (float)(sx - x0);
            tfy = (float)(sy - y0);
        }
        float wx[4], wy[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            wx[q] = cubic_wf(tfx + 1.f - (float)q);
            wy[q] = cubic_wf(tfy + 1.f - (float)q);
        }
        // plane order for interpolation: Px Py Pxx Pyy Pxy Hx Hxx Hxy Hyy Hy
        float v[10];
#pragma unroll
        for (int pl = 0; pl < 10; ++pl) v[pl] = 0.f;
#pragma unroll
        for (int pp = 0; pp < 4; ++pp) {
            int ii = y0 - 1 + pp;
            ii = ii < 0 ? 0 : (ii >= h ? h - 1 : ii);
            const int ra = ii - (i0 - HB);           // row in the conv region
            const int rin = ii - ri;                 // row in the input region
            float rowv[10];
#pragma unroll
            for (int pl = 0; pl < 10; ++pl) rowv[pl] = 0.f;
#pragma unroll
            for (int qq = 0; qq < 4; ++qq) {
                int jj = x0 - 1 + qq;
                jj = jj < 0 ? 0 : (jj >= w ? w - 1 : jj);
                const int ca = jj - (j0 - HB);
                const int cin = jj - rj;
                const int o = ra * NO + ca;
                const float wq = wx[qq];
                rowv[0] = fmaf(sColA[0 * NO * NO + o], wq, rowv[0]);
                rowv[1] = fmaf(sColA[1 * NO * NO + o], wq, rowv[1]);
                rowv[2] = fmaf(sColA[2 * NO * NO + o], wq, rowv[2]);
                rowv[3] = fmaf(sColA[4 * NO * NO + o], wq, rowv[3]);
                rowv[4] = fmaf(sColA[3 * NO * NO + o], wq, rowv[4]);
                rowv[5] = fmaf(sHx[rin * NI + cin], wq, rowv[5]);
                rowv[6] = fmaf(sColB[0 * NO * NO + o], wq, rowv[6]);
                rowv[7] = fmaf(sColB[2 * NO * NO + o], wq, rowv[7]);
                rowv[8] = fmaf(sColB[1 * NO * NO + o], wq, rowv[8]);
                rowv[9] = fmaf(sHy[rin * NI + cin], wq, rowv[9]);
            }
#pragma unroll
            for (int pl = 0; pl < 10; ++pl) v[pl] = fmaf(rowv[pl], wy[pp], v[pl]);
        }
        float ori;
        float Fx, Fy;
        // plane order: Px Py Pxx Pyy Pxy Hx Hxx Hxy Hyy Hy (:683-684)
        if (p.hyb) {
            Fx = dot4_comp(v[0], v[6], v[2], v[5], v[1], v[7], v[4], v[9]);  // Px Hxx + Pxx Hx + Py Hxy + Pxy Hy
            Fy = dot4_comp(v[0], v[7], v[4], v[5], v[1], v[8], v[3], v[9]);  // Px Hxy + Pxy Hx + Py Hyy + Pyy Hy
        } else {
            Fx = v[0] * v[6] + v[2] * v[5] + v[1] * v[7] + v[4] * v[9];
            Fy = v[0] * v[7] + v[4] * v[5] + v[1] * v[8] + v[3] * v[9];
        }
        // |F| < 1e-12: the NMS direction instead (:686-690); otherwise the
        // angle of F itself (atan2 of the normalised vector is that of F)
        if (fmaf(Fx, Fx, Fy * Fy) < 1e-24f) {
            const int pi = p.sc.staging_idx[sidx];
            const float2 d = p.dir[M.px_base + pi];
            ori = atan2f(d.x, -d.y);
        } else {
            ori = atan2f(Fx, -Fy);
        }
        rec.z = (double)ori;
        // coord_scale (:657, :696-697): positions in original pixels
        rec.x = sx * inv_scale;
        rec.y = sy * inv_scale;
        p.sc.staging[sidx] = rec;
    }
}

// ---------------------------------------------------------------------------
// Isolated-edgel removal (:563-621) and stable compaction
// ---------------------------------------------------------------------------
// segment tile t -> (map, first local segment)
__device__ __forceinline__ int seg_map(const SubParams& p, int t)
{
    return find_image(p.n_maps, t, [&](int i) { return p.m[i].seg_tile_base; });
}

// One CTA per tile of kSegTile segments, a thread per staged edgel of the
// tile (owning segment by binary search over the scanned counts): an edgel
// survives if another lies within the radius and in its 3x3 cell
// neighbourhood (:563-621).  Candidates come from the per-pixel id map,
// searched ring by ring from the edgel's own pixel outwards and stopping at
// the first hit (the result does not depend on the order).
__global__ void __launch_bounds__(256) tc_isolate(const __grid_constant__ SubParams p)
{
    constexpr int PER = kSegTile / 256;
    __shared__ int s_warp[33];
    __shared__ int s_dst[kSegTile];  // exclusive prefix of segment counts within the tile
    __shared__ int s_src[kSegTile];  // staging offset of each segment
    const int t = blockIdx.x;
    const int k = seg_map(p, t);
    const SubMap& M = p.m[k];
    const long long nseg = (long long)M.h * M.ntx;
    const long long q0 = (long long)(t - M.seg_tile_base) * kSegTile + threadIdx.x * PER;
    int cnt[PER], sum = 0;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int2 sg = (q0 + u < nseg) ? p.sc.seg[M.seg_base + q0 + u] : make_int2(0, 0);
        cnt[u] = sg.y;
        s_src[threadIdx.x * PER + u] = sg.x;
        sum += sg.y;
    }
    int total;
    int run = block_excl_scan<256>(sum, s_warp, &total);
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        s_dst[threadIdx.x * PER + u] = run;
        run += cnt[u];
    }
    __syncthreads();
    const bool all = !(p.nbr > 0.0) || p.img_count[k] < 2;  // :567-568
    const double r2 = p.nbr * p.nbr;
    // an edgel lies within sqrt(2) work pixels of its own; search the id map
    // (work grid) around it, compare in original pixels as the reference does
    const int reach = (int)ceil(p.nbr * M.scale + 1.5);
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int lo = 0, hi = kSegTile - 1;  // last segment with s_dst <= e
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_dst[mid] <= e) lo = mid; else hi = mid - 1;
        }
        const long long r = (long long)s_src[lo] + (e - s_dst[lo]);
        if (r >= p.sc.staging_cap) continue;
        if (all) {
            p.keep[r] = 1;
            continue;
        }
        const double4_32a me = p.sc.staging[r];
        const int pi = (int)floor(me.y * M.scale), pj = (int)floor(me.x * M.scale);
        bool found = false;
        for (int d = 0; d <= reach && !found; ++d) {
            for (int ii = pi - d; ii <= pi + d && !found; ++ii) {
                if (ii < 0 || ii >= M.h) continue;
                const int step = (ii == pi - d || ii == pi + d) ? 1 : 2 * d;  // ring: full edge rows, end columns
                for (int jj = pj - d; jj <= pj + d; jj += step) {
                    if (jj < 0 || jj >= M.w) continue;
                    const int o = p.eid[M.px_base + (long long)ii * M.w + jj];
                    if (o < 0 || o == r) continue;
                    // the reference looks only in the 3 x 3 cells of size radius
                    // around the edgel's cell; every edgel within the radius
                    // lies in one of them, so the distance test alone decides
                    const double4_32a ot = p.sc.staging[o];
                    const double ddx = me.x - ot.x, ddy = me.y - ot.y;
                    if (ddx * ddx + ddy * ddy <= r2) {
                        found = true;
                        break;
                    }
                }
            }
        }
        p.keep[r] = found ? 1 : 0;
    }
}

__global__ void __launch_bounds__(256) tc_compact(const __grid_constant__ SubParams p)
{
    const int t = blockIdx.x;
    const int k = seg_map(p, t);
    const SubMap& M = p.m[k];
    const long long nseg = (long long)M.h * M.ntx;
    for (int q = threadIdx.x; q < kSegTile; q += blockDim.x) {
        const long long local = (long long)(t - M.seg_tile_base) * kSegTile + q;
        if (local >= nseg) break;
        int2 sg = p.sc.seg[M.seg_base + local];
        long long wpos = sg.x;
        for (int e = 0; e < sg.y; ++e) {
            const long long r = (long long)sg.x + e;
            if (r >= p.sc.staging_cap) break;
            if (p.keep[r]) {
                if (wpos != r) {
                    p.sc.staging[wpos] = p.sc.staging[r];
                    p.sc.staging_idx[wpos] = p.sc.staging_idx[r];
                }
                ++wpos;
            }
        }
        sg.y = (int)(wpos - sg.x);
        p.sc.seg[M.seg_base + local] = sg;
    }
}

// Dense TO_E / TO_O (:708-715): pass 0 elects, per pixel, the last edgel in
// list order that rounds onto it; pass 1 writes its strength and orientation.
template <int PASS>
__global__ void __launch_bounds__(kSegTile) tc_dense(const __grid_constant__ SubParams p)
{
    __shared__ int s_warp[33];
    const int t = blockIdx.x;
    const int k = seg_map(p, t);
    const SubMap& M = p.m[k];
    const long long nseg = (long long)M.h * M.ntx;
    const long long local = (long long)(t - M.seg_tile_base) * kSegTile + threadIdx.x;
    const int2 sg = (local < nseg) ? p.sc.seg[M.seg_base + local] : make_int2(0, 0);
    // block-wide exclusive scan of the segment counts (same order as the ordering pass)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = sg.y;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int v = s_warp[lane];
        int wi = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        s_warp[lane] = wi - v;
    }
    __syncthreads();
    if (M.TO_E == nullptr && M.TO_O == nullptr) return;
    const long long dest = (long long)p.sc.tile_sum[t] + (incl - sg.y + s_warp[wid]) - p.sc.img_base[k];
    for (int e = 0; e < sg.y; ++e) {
        const long long r = (long long)sg.x + e;
        if (r >= p.sc.staging_cap) break;
        const double4_32a rec = p.sc.staging[r];
        int X = (int)round(rec.x), Y = (int)round(rec.y);
        X = max(0, min(X, M.ow - 1));
        Y = max(0, min(Y, M.oh - 1));
        const long long o = (long long)Y * M.ow + X;  // original grid (also indexes the winner map)
        const int li = (int)(dest + e);
        if (PASS == 0) {
            atomicMax(&p.win[M.px_base + o], li);
        } else if (p.win[M.px_base + o] == li) {
            if (p.out_f64) {
                if (M.TO_E) reinterpret_cast<double*>(M.TO_E)[o] = rec.w;
                if (M.TO_O) reinterpret_cast<double*>(M.TO_O)[o] = rec.z;
            } else {
                if (M.TO_E) reinterpret_cast<float*>(M.TO_E)[o] = (float)rec.w;
                if (M.TO_O) reinterpret_cast<float*>(M.TO_O)[o] = (float)rec.z;
            }
        }
    }
}

// bilinear_resize (:69-90) of one map onto the work grid, in FP64.
__global__ void __launch_bounds__(256) tc_resize(const void* __restrict__ src, int dtype, long long pitch, int sh,
                                                 int sw, double* __restrict__ dst, int dh, int dw)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= dw || i >= dh) return;
    auto at = [&](int y, int x) -> double {
        const long long o = (long long)y * pitch + x;
        return dtype == TOED_F64 ? __ldg((const double*)src + o) : (double)__ldg((const float*)src + o);
    };
    const double y = (dh == 1) ? 0.0 : (double)i * (sh - 1) / (double)(dh - 1);
    const int y0 = (int)floor(y), y1 = min(y0 + 1, sh - 1);
    const double fy = y - y0;
    const double x = (dw == 1) ? 0.0 : (double)j * (sw - 1) / (double)(dw - 1);
    const int x0 = (int)floor(x), x1 = min(x0 + 1, sw - 1);
    const double fx = x - x0;
    const double v00 = at(y0, x0), v01 = at(y0, x1), v10 = at(y1, x0), v11 = at(y1, x1);
    dst[(long long)i * dw + j] = (1 - fy) * ((1 - fx) * v00 + fx * v01) + fy * ((1 - fx) * v10 + fx * v11);
}

template <int R>
static const void* correct_kernel() { return (const void*)tc_correct<R>; }

static const void* correct_entry(int r, size_t* smem)
{
    switch (r) {
#define TOED_TC_CASE(R) \
    case R: *smem = CorrCfg<R>::smem; return correct_kernel<R>();
        TOED_TC_CASE(1) TOED_TC_CASE(2) TOED_TC_CASE(3) TOED_TC_CASE(4) TOED_TC_CASE(5) TOED_TC_CASE(6)
        TOED_TC_CASE(7) TOED_TC_CASE(8) TOED_TC_CASE(9) TOED_TC_CASE(10) TOED_TC_CASE(11) TOED_TC_CASE(12)
#undef TOED_TC_CASE
    default: return nullptr;
    }
}

// Host side of toed_subpix_to_correct_batch for one chunk of maps.
cudaError_t subpix_launch(const toed_edgemap* maps, int n, const toed_subpix_params* prm, int r,
                          const SubScratch& s, cudaStream_t stream)
{
    SubParams* p = new SubParams();
    std::memset(p, 0, sizeof(SubParams));
    const double sig = prm->sigma, s2 = sig * sig, s3 = s2 * sig, s5 = s2 * s3;
    const double nrm = std::sqrt(2.0 * 3.14159265358979323846);
    for (int kk = -r; kk <= r; ++kk) {  // build_gaussian_kernels :207-213
        const double x = kk, e = std::exp(-(x * x) / (2.0 * s2));
        p->g[0][kk + r] = (float)(e / (nrm * sig));
        p->g[1][kk + r] = (float)(-x * e / (nrm * s3));
        p->g[2][kk + r] = (float)((x * x - s2) * e / (nrm * s5));
    }
    p->r = r;
    p->thresh = prm->thresh;
    p->nbr = prm->nbr_radius;
    p->hyb = prm->precision != TOED_FP32;
    p->out_f64 = prm->out_dtype == TOED_F64;
    p->n_maps = n;
    const int sc = 1 << prm->interp_n;
    long long px = 0, segtiles = 0, work = 0;
    int tiles = 0;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < n; ++i) {
        const toed_edgemap& m = maps[i];
        SubMap& d = p->m[i];
        d.oh = m.height;
        d.ow = m.width;
        d.scale = sc;
        d.margin = 3 * sc;
        d.h = (m.height - 1) * sc + 1;
        d.w = (m.width - 1) * sc + 1;
        if (sc == 1) {
            d.E = m.E;
            d.theta = m.theta;
            d.pitch = m.pitch;
            d.dtype = m.dtype;
        } else {  // set_edgemap / set_orientation (:224-244): resize onto the work grid
            const long long hw = (long long)d.h * d.w;
            double* wE = s.work + work;
            work += hw;
            const dim3 g((d.w + 255) / 256, d.h);
            tc_resize<<<g, 256, 0, stream>>>(m.E, m.dtype, m.pitch, m.height, m.width, wE, d.h, d.w);
            d.E = wE;
            d.theta = nullptr;
            if (m.theta) {
                double* wT = s.work + work;
                work += hw;
                tc_resize<<<g, 256, 0, stream>>>(m.theta, m.dtype, m.pitch, m.height, m.width, wT, d.h, d.w);
                d.theta = wT;
            }
            d.pitch = d.w;
            d.dtype = TOED_F64;
            if (e == cudaSuccess) e = cudaGetLastError();
        }
        d.px_base = px;
        d.TO_E = m.TO_E;
        d.TO_O = m.TO_O;
        d.ntx = (d.w + kT - 1) / kT;
        d.nty = (d.h + kT - 1) / kT;
        d.tile_base = tiles;
        d.seg_tile_base = (int)segtiles;
        d.seg_base = segtiles * kSegTile;
        const long long nseg = (long long)d.h * d.ntx;
        tiles += d.ntx * d.nty;
        segtiles += (nseg + kSegTile - 1) / kSegTile;
        px += (long long)d.h * d.w;
    }
    p->n_tiles = tiles;
    p->n_seg_tiles = (int)segtiles;
    p->sc = s.sc;
    p->dir = s.dir;
    p->eid = s.eid;
    p->win = s.win;
    p->img_count = s.img_count;
    p->keep = s.keep;
    std::unique_ptr<SubParams> guard(p);

    if (e == cudaSuccess) e = cudaMemsetAsync(s.sc.words, 0, 3 * sizeof(int), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.img_count, 0, sizeof(int) * n, stream);
    void* args[] = {p};
    if (e == cudaSuccess) e = cudaLaunchKernel((const void*)tc_orient_nms, dim3(tiles), dim3(256), args, 0, stream);
    size_t smem = 0;
    const void* cf = correct_entry(r, &smem);
    if (!cf) return cudaErrorInvalidValue;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(cf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaLaunchKernel(cf, dim3(tiles), dim3(512), args, smem, stream);
    if (e == cudaSuccess) e = cudaLaunchKernel((const void*)tc_isolate, dim3(p->n_seg_tiles), dim3(256), args, 0, stream);
    if (e == cudaSuccess) e = cudaLaunchKernel((const void*)tc_compact, dim3(p->n_seg_tiles), dim3(256), args, 0, stream);
    // ordering pass shared with the detector
    BatchParams* b = new BatchParams();
    std::memset(b, 0, sizeof(BatchParams));
    std::unique_ptr<BatchParams> bguard(b);
    b->n_img = n;
    b->n_tiles = p->n_seg_tiles;
    b->out_f64 = p->out_f64;
    b->sc = s.sc;
    for (int i = 0; i < n; ++i) {
        DetImage& d = b->img[i];
        d.out = maps[i].edgels;
        d.count = maps[i].count;
        d.index = nullptr;
        d.seg_base = p->m[i].seg_base;
        d.nseg = (long long)p->m[i].h * p->m[i].ntx;
        d.tile_base = p->m[i].seg_tile_base;
        d.cap = maps[i].capacity;
        d.H = p->m[i].h;
        d.W = p->m[i].w;
    }
    if (e == cudaSuccess) e = launch_finalize(*b, stream);
    bool dense = false;
    for (int i = 0; i < n; ++i) dense = dense || maps[i].TO_E || maps[i].TO_O;
    if (dense && e == cudaSuccess) {
        e = cudaMemsetAsync(s.win, 0xff, sizeof(int) * (size_t)px, stream);
        const size_t es = p->out_f64 ? sizeof(double) : sizeof(float);
        for (int i = 0; i < n && e == cudaSuccess; ++i) {
            const size_t bytes = es * (size_t)maps[i].height * maps[i].width;
            if (maps[i].TO_E) e = cudaMemsetAsync(maps[i].TO_E, 0, bytes, stream);
            if (e == cudaSuccess && maps[i].TO_O) e = cudaMemsetAsync(maps[i].TO_O, 0, bytes, stream);
        }
        if (e == cudaSuccess)
            e = cudaLaunchKernel((const void*)tc_dense<0>, dim3(p->n_seg_tiles), dim3(kSegTile), args, 0, stream);
        if (e == cudaSuccess)
            e = cudaLaunchKernel((const void*)tc_dense<1>, dim3(p->n_seg_tiles), dim3(kSegTile), args, 0, stream);
    }
    return e;
}

}  // namespace toed
