// toed_qad.cu -- the MATLAB "quick and dirty" orientation mode
// (third_order_edge_detector.m:91-141 with QaD_flag set), as the last kernel
// of the ordering pass.
//
// In this mode the emitted orientation is the third-order direction
// atan2(Fx, -Fy) (:127-141) built from the nine derivatives interpolated
// with MATLAB's interp2 'cubic' -- cubic convolution, Keys a = -1/2, the
// kernel the reference also restates as cubic_kernel
// (subpix_to_correction.cpp:57-67) -- at the edgel's subpixel point, instead
// of the direction at its 2x-grid point (cpu_toed.cpp:227-232).  The
// derivatives are the C++ detector's own (2x grid, zero padding,
// cpu_toed.cpp:204-344); positions and strengths are unchanged.
//
// fin_scatter_qad<R> replaces fin_scatter: per tile of segments the same
// scan, then a warp per staged edgel
//   1. takes the subpixel point pos = 2 x_out + 1 (FP64, cpu_toed.cpp:516)
//      and the 4 x 4 block of 2x-grid points around it with their Keys
//      weights;
//   2. loads the (2r+5) x (2r+5) window of image pixels that all sixteen
//      points' filters cover -- lane c holds window column c, rows loaded
//      coalesced;
//   3. folds the block's four columns into three weighted x-tap vectors
//      per lane (interpolation is linear), contracts the window column with
//      each point row's y taps (lane-local) and accumulates the nine
//      interpolated derivatives;
//   4. sums the nine values over the lanes (butterfly) and parks them; after
//      32 records lane e forms record e's third-order vector, the angle and
//      the output record; in HYBRID precision the records whose vector nearly
//      cancels are first contracted again in FP64 by the whole warp.
#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

namespace {

constexpr int kQadThreads = 128;
constexpr int kQadSegPerThread = kSegTile / kQadThreads;

// Keys cubic convolution kernel, a = -1/2 (subpix_to_correction.cpp:57-67).
template <typename T>
__device__ __forceinline__ T keys(T s)
{
    const T a = T(-0.5), x = fabs(s);
    if (x <= T(1)) return ((a + T(2)) * x - (a + T(3))) * x * x + T(1);
    if (x < T(2)) return ((a * x - T(5) * a) * x + T(8) * a) * x - T(4) * a;
    return T(0);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// Four filter values (G, Gx, Gxx, Gxxx) in FP32 (float4) or FP64 (double4_32a).
template <typename T> struct Vec4;
template <> struct Vec4<float> {
    using type = float4;
    static __device__ __forceinline__ float4 make(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
};
template <> struct Vec4<double> {
    using type = double4_32a;
    static __device__ __forceinline__ double4_32a make(double a, double b, double c, double d)
    {
        return make_double4_32a(a, b, c, d);
    }
};

}  // namespace

// The nine derivatives of one (x taps, y contraction) pairing, added in:
// x = (G, Gx, Gxx, Gxxx) taps of this lane's column (weighted), c = the
// column's contractions with (G, Gy, Gyy, Gyyy).
template <typename T, typename V>
__device__ __forceinline__ void qad_pair(V x, V c, T (&acc)[9])
{
    acc[0] = fma(x.y, c.x, acc[0]);  // fx   = Gx   (x) G
    acc[1] = fma(x.x, c.y, acc[1]);  // fy   = G    (x) Gy
    acc[2] = fma(x.z, c.x, acc[2]);  // fxx  = Gxx  (x) G
    acc[3] = fma(x.y, c.y, acc[3]);  // fxy  = Gx   (x) Gy
    acc[4] = fma(x.x, c.z, acc[4]);  // fyy  = G    (x) Gyy
    acc[5] = fma(x.z, c.y, acc[5]);  // fxxy = Gxx  (x) Gy
    acc[6] = fma(x.y, c.z, acc[6]);  // fxyy = Gx   (x) Gyy
    acc[7] = fma(x.w, c.x, acc[7]);  // fxxx = Gxxx (x) G
    acc[8] = fma(x.x, c.w, acc[8]);  // fyyy = G    (x) Gyyy
}

template <typename T, typename V>
__device__ __forceinline__ V v4_fma(T a, V x, V y)
{
    return Vec4<T>::make(fma(a, x.x, y.x), fma(a, x.y, y.y), fma(a, x.z, y.z), fma(a, x.w, y.w));
}

template <typename T, typename V>
__device__ __forceinline__ V v4_scale(T a, V x) { return Vec4<T>::make(a * x.x, a * x.y, a * x.z, a * x.w); }

// Interpolation is linear, so the four columns of the 4 x 4 block fold into
// three weighted x-tap vectors per lane, one per x variant in use: columns
// of parity b = 0 take T taps in rows of parity a = 0 and F taps in rows
// a = 1; columns b = 1 take S taps.  The columns' parities alternate from
// X1 - 1, so B0 (0 or 1) is the parity of the block's first column.
template <int R, int B0, typename T, typename V>
__device__ __forceinline__ void qad_columns(const V* __restrict__ sTab, int X1, int j, int l, const T (&wx)[4],
                                            V& xT, V& xF, V& xS)
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4;
    xT = xF = xS = Vec4<T>::make(T(0), T(0), T(0), T(0));
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int dj = ((X1 - 1 + s) >> 1) - j;
        const int e = NT + 2 + dj - l;  // padded entry of this lane's column
        if (((B0 + s) & 1) == 0) {
            xT = v4_fma(wx[s], sTab[e], xT);
            xF = v4_fma(wx[s], sTab[NTP + e], xF);
        } else {
            xS = v4_fma(wx[s], sTab[2 * NTP + e], xS);
        }
    }
}

// One row of the 4 x 4 block: 2x-grid row parity A, original row offset DI
// from the window centre (both fixed by the parity of the block's first row).
// Contracts this lane's window column with the row's y taps -- shifted (S)
// for A = 1; full (F) for A = 0, the truncated set (T) being F without its
// two end taps -- weights it by the row's Keys weight and adds the row's
// sub-grids: (0,0) T x T, (0,1) S x F, (1,0) F x S, (1,1) S x S (x by y).
template <int R, int A, int DI, typename T, typename V>
__device__ __forceinline__ void qad_row(const float (&v)[2 * R + 5], const V* __restrict__ sTab, T wy, V xT, V xF,
                                        V xS, T (&acc)[9])
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4, NU = NT + 2;
    const V* Yt = sTab + (A ? 2 : 1) * NTP + NT + 2 + DI;  // entry NT + 2 + DI - u: tap of window row u
    V c = Vec4<T>::make(T(0), T(0), T(0), T(0));
#pragma unroll
    for (int u = 0; u < NU; ++u) {
        const V y = Yt[-u];
        const T x = v[u];
        c.x = fma(x, y.x, c.x); c.y = fma(x, y.y, c.y);
        c.z = fma(x, y.z, c.z); c.w = fma(x, y.w, c.w);
    }
    if (A) {
        const V cs = v4_scale(wy, c);
        qad_pair(xF, cs, acc);
        qad_pair(xS, cs, acc);
    } else {
        // T = F less the taps k = 0 (window row NT + DI) and k = NT - 1 (window row DI + 1)
        const V e0 = sTab[NTP + 2], e1 = sTab[NTP + 2 + NT - 1];
        const T va = v[NT + DI], vb = v[DI + 1];
        V t;
        t.x = fma(-vb, e1.x, fma(-va, e0.x, c.x));
        t.y = fma(-vb, e1.y, fma(-va, e0.y, c.y));
        t.z = fma(-vb, e1.z, fma(-va, e0.z, c.z));
        t.w = fma(-vb, e1.w, fma(-va, e0.w, c.w));
        qad_pair(xT, v4_scale(wy, t), acc);
        qad_pair(xS, v4_scale(wy, c), acc);
    }
}

// The nine derivatives interpolated at subpixel point (X1 + tx, Y1 + ty) of
// the 2x grid from this lane's window column v: step 1 (Keys weights) and
// step 3 of the file comment, before the sum over lanes.
template <int R, typename T>
__device__ __forceinline__ void qad_point(const float (&v)[2 * R + 5], const typename Vec4<T>::type* __restrict__ sTab,
                                          int X1, int Y1, T tx, T ty, int l, T (&acc)[9])
{
    using V = typename Vec4<T>::type;
    const int j = X1 >> 1;
    T wx[4], wy[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        wx[s] = keys(tx + T(1) - (T)s);
        wy[s] = keys(ty + T(1) - (T)s);
    }
    V xT, xF, xS;
    if ((X1 & 1) == 0)
        qad_columns<R, 1>(sTab, X1, j, l, wx, xT, xF, xS);
    else
        qad_columns<R, 0>(sTab, X1, j, l, wx, xT, xF, xS);
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] = T(0);
    if ((Y1 & 1) == 0) {
        qad_row<R, 1, -1>(v, sTab, wy[0], xT, xF, xS, acc);
        qad_row<R, 0, 0>(v, sTab, wy[1], xT, xF, xS, acc);
        qad_row<R, 1, 0>(v, sTab, wy[2], xT, xF, xS, acc);
        qad_row<R, 0, 1>(v, sTab, wy[3], xT, xF, xS, acc);
    } else {
        qad_row<R, 0, 0>(v, sTab, wy[0], xT, xF, xS, acc);
        qad_row<R, 1, 0>(v, sTab, wy[1], xT, xF, xS, acc);
        qad_row<R, 0, 1>(v, sTab, wy[2], xT, xF, xS, acc);
        qad_row<R, 1, 1>(v, sTab, wy[3], xT, xF, xS, acc);
    }
}

// The third-order vector (cpu_toed.cpp:227-232) in FP64 from nine derivatives.
template <typename T>
__device__ __forceinline__ void to_vector(const T (&d)[9], double& tix, double& tiy)
{
    const double fx = d[0], fy = d[1], fxx = d[2], fxy = d[3], fyy = d[4], fxxy = d[5], fxyy = d[6],
                 fxxx = d[7], fyyy = d[8];
    tix = fx * (2.0 * fxx * fxx + 2.0 * fxy * fxy) + fy * (2.0 * fxx * fxy + 2.0 * fyy * fxy) +
          2.0 * fx * fy * fxxy + fy * fy * fxyy + fx * fx * fxxx;
    tiy = fx * (2.0 * fxx * fxy + 2.0 * fyy * fxy) + fy * (2.0 * fyy * fyy + 2.0 * fxy * fxy) +
          2.0 * fx * fy * fxyy + fx * fx * fxxy + fy * fy * fyyy;
}

// FP64 pass for one record (the whole warp): the window around the record's
// subpixel point (2x-grid coordinates px, py), the interpolated derivatives
// with FP64 weights and taps, their sum over the lanes and the third-order
// vector (every lane gets it).  Out of line: it is rare, and inlined its
// registers would crowd the FP32 contraction.
template <int R>
__device__ __noinline__ double2 qad_refine(const void* src, long long pitch, int H, int W, bool u8,
                                           const double4_32a* __restrict__ sTab64, double px, double py, int lane)
{
    constexpr int NU = 2 * R + 5;
    const double fpx = floor(px), fpy = floor(py);
    const int X1 = (int)fpx, Y1 = (int)fpy;
    const int i = Y1 >> 1, col = (X1 >> 1) - R - 2 + lane;
    const bool okc = lane < NU && col >= 0 && col < W;
    float w[NU];
#pragma unroll
    for (int u = 0; u < NU; ++u) {
        const int y = i - R - 2 + u;
        w[u] = 0.f;
        if (okc && (unsigned)y < (unsigned)H) {
            const long long o = (long long)y * pitch + col;
            w[u] = u8 ? (float)static_cast<const unsigned char*>(src)[o] : static_cast<const float*>(src)[o];
        }
    }
    double acc[9];
    qad_point<R, double>(w, sTab64, X1, Y1, px - fpx, py - fpy, lane < NU ? lane : NU - 1, acc);
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] = warp_sum(acc[q]);
    double2 ti;
    to_vector(acc, ti.x, ti.y);
    return ti;
}

template <int R>
__global__ void __launch_bounds__(kQadThreads, 3) fin_scatter_qad(const __grid_constant__ BatchParams p)
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4, NU = NT + 2;
    static_assert(NU <= 32, "one lane per window column");
    __shared__ int s_warp[33];
    __shared__ int s_dst[kSegTile];
    __shared__ int s_src[kSegTile];
    // taps per variant T (2r+1, ends zero) / F (2r+3) / S (shifted): (G, Gx, Gxx, Gxxx), two zero entries
    // each side, so that entry NT + 2 + d - c is the tap of window row / column c for a point at offset d
    __shared__ float4 sTab[3 * NTP];
    // the same in FP64 (HYBRID precision: records whose third-order vector nearly cancels)
    __shared__ double4_32a sTab64[3 * NTP];
    // per warp, the nine derivatives of the 32 records in flight (stride 9: conflict-free per lane)
    __shared__ float sDer[kQadThreads / 32][32 * 9];
    for (int i = threadIdx.x; i < 3 * NTP; i += kQadThreads) {
        const int v = i / NTP, k = i - v * NTP - 2;
        const int f = (v == 2) ? 4 : 0;
        float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
        double4_32a t64 = make_double4_32a(0.0, 0.0, 0.0, 0.0);
        if (k >= 0 && k < NT && !(v == 0 && (k == 0 || k == NT - 1))) {
            t = make_float4(p.taps.v[f][k], p.taps.v[f + 1][k], p.taps.v[f + 2][k], p.taps.v[f + 3][k]);
            t64 = make_double4_32a(p.taps64.v[f][k], p.taps64.v[f + 1][k], p.taps64.v[f + 2][k],
                                   p.taps64.v[f + 3][k]);
        }
        sTab[i] = t;
        sTab64[i] = t64;
    }
    const int t = blockIdx.x;
    const int k = find_image(p.n_img, t, [&](int i) { return p.img[i].tile_base; });
    const DetImage& im = p.img[k];
    const long long q0 = (long long)(t - im.tile_base) * kSegTile + threadIdx.x * kQadSegPerThread;
    int cnt[kQadSegPerThread], sum = 0;
#pragma unroll
    for (int u = 0; u < kQadSegPerThread; ++u) {
        const long long q = q0 + u;
        const int2 sg = (q < im.nseg) ? p.sc.seg[im.seg_base + q] : make_int2(0, 0);
        cnt[u] = sg.y;
        s_src[threadIdx.x * kQadSegPerThread + u] = sg.x;
        sum += sg.y;
    }
    int total;
    int run = block_excl_scan<kQadThreads>(sum, s_warp, &total);
#pragma unroll
    for (int u = 0; u < kQadSegPerThread; ++u) {
        s_dst[threadIdx.x * kQadSegPerThread + u] = run;
        run += cnt[u];
    }
    __syncthreads();
    const long long base = (long long)p.sc.tile_sum[t] - p.sc.img_base[k];
    const long long cap = im.cap;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int l = lane < NU ? lane : NU - 1;  // lanes past the window repeat its last column (their pixels are 0)
    // each warp takes 32 consecutive records: their derivatives one after
    // another (all lanes), then lane e finishes record e (FP64 with all lanes busy)
    for (int r0 = wid * 32; r0 < total; r0 += kQadThreads) {
        // lane e locates record r0 + e (list position, staging slot) and its
        // subpixel point pos = 2 x_out + 1 on the 2x grid (cpu_toed.cpp:516)
        int my_d = -1, mX1 = 0, mY1 = 0;
        long long my_src = 0;
        float mtx = 0.f, mty = 0.f;
        if (r0 + lane < total) {
            const int r = r0 + lane;
            int lo = 0, hi = kSegTile - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_dst[mid] <= r) lo = mid; else hi = mid - 1;
            }
            const long long d = base + r, src = (long long)s_src[lo] + (r - s_dst[lo]);
            if (d < cap && src < p.sc.staging_cap) {
                const double2 xy = det_xy(det_stage(p.sc)[src], p.sc.staging_idx[src], 2 * im.W, p.hyb != 0);
                const double px = 2.0 * xy.x + 1.0, py = 2.0 * xy.y + 1.0;
                const double fpx = floor(px), fpy = floor(py);
                mX1 = (int)fpx;
                mY1 = (int)fpy;
                mtx = (float)(px - fpx);
                mty = (float)(py - fpy);
                my_d = (int)d;
                my_src = src;
            }
        }
        const int ne = min(32, total - r0);
        // the window around the original pixel (Y1 >> 1, X1 >> 1) of record e's
        // grid point, one column per lane; the next record's window is loaded
        // while this one is reduced (records past the capacity read a window
        // that is computed on and dropped)
        auto load_window = [&](int e, float (&w)[NU]) {
            const int Xe = __shfl_sync(0xffffffffu, mX1, e), Ye = __shfl_sync(0xffffffffu, mY1, e);
            const int i = Ye >> 1, col = (Xe >> 1) - R - 2 + lane;
            const bool okc = lane < NU && col >= 0 && col < im.W;
            if (im.dtype == TOED_U8) {
                const unsigned char* sp = (const unsigned char*)im.src + col;
#pragma unroll
                for (int u = 0; u < NU; ++u) {
                    const int y = i - R - 2 + u;
                    w[u] = (okc && (unsigned)y < (unsigned)im.H) ? (float)__ldg(sp + (long long)y * im.pitch) : 0.f;
                }
            } else {
                const float* sp = (const float*)im.src + col;
#pragma unroll
                for (int u = 0; u < NU; ++u) {
                    const int y = i - R - 2 + u;
                    w[u] = (okc && (unsigned)y < (unsigned)im.H) ? __ldg(sp + (long long)y * im.pitch) : 0.f;
                }
            }
        };
        float vn[NU];
        load_window(0, vn);
        for (int e = 0; e < ne; ++e) {
            float v[NU];
#pragma unroll
            for (int u = 0; u < NU; ++u) v[u] = vn[u];
            if (e + 1 < ne) load_window(e + 1, vn);
            const int X1 = __shfl_sync(0xffffffffu, mX1, e), Y1 = __shfl_sync(0xffffffffu, mY1, e);
            const float tx = __shfl_sync(0xffffffffu, mtx, e), ty = __shfl_sync(0xffffffffu, mty, e);
            float acc[9];
            qad_point<R, float>(v, sTab, X1, Y1, tx, ty, l, acc);
            // 4. sums over the window columns, parked for lane e
#pragma unroll
            for (int q = 0; q < 9; ++q) acc[q] = warp_sum(acc[q]);
            if (lane == 0) {
#pragma unroll
                for (int q = 0; q < 9; ++q) sDer[wid][e * 9 + q] = acc[q];
            }
        }
        __syncwarp();
        float mine[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) mine[q] = sDer[wid][lane * 9 + q];
        __syncwarp();  // the next group overwrites the slots
        const float4 my_st = my_d >= 0 ? det_stage(p.sc)[my_src] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int my_gi = my_d >= 0 ? p.sc.staging_idx[my_src] : 0;
        const double2 my_xy = my_d >= 0 ? det_xy(my_st, my_gi, 2 * im.W, p.hyb != 0) : make_double2(0.0, 0.0);
        // the third-order vector and the angle
        const float gx = mine[0], gy = mine[1], fxx = mine[2], fxy = mine[3], fyy = mine[4], fxxy = mine[5],
                    fxyy = mine[6], fxxx = mine[7], fyyy = mine[8];
        float ori;
        if (p.hyb) {
            // FP32 vector; the ill-conditioned ones are redone in FP64 below
            const float a2 = fmaf(fxx, fxx, fxy * fxy), c2 = fmaf(fyy, fyy, fxy * fxy), bc = fxy * (fxx + fyy);
            const float pxy = gx * gy, x2 = gx * gx, y2 = gy * gy;
            double tix = fmaf(2.f, fmaf(gx, a2, fmaf(gy, bc, pxy * fxxy)), fmaf(y2, fxyy, x2 * fxxx));
            double tiy = fmaf(2.f, fmaf(gx, bc, fmaf(gy, c2, pxy * fxyy)), fmaf(x2, fxxy, y2 * fyyy));
            // Records whose vector cancels by more than kRefineKappa (sum of
            // the terms' magnitudes over the largest component) carry the FP32
            // contraction's rounding multiplied by that ratio: the warp
            // recomputes their nine derivatives in FP64, one record at a time.
            const float ax = fabsf(gx), ay = fabsf(gy), pxx = fabsf(fxx * fxy), pyy = fabsf(fyy * fxy);
            const float sabs = 2.f * ax * (fxx * fxx + fxy * fxy) + 2.f * ay * (fyy * fyy + fxy * fxy) +
                               2.f * (ax + ay) * (pxx + pyy) + 2.f * ax * ay * (fabsf(fxxy) + fabsf(fxyy)) +
                               ay * ay * (fabsf(fxyy) + fabsf(fyyy)) + ax * ax * (fabsf(fxxx) + fabsf(fxxy));
            const float tmax = fmaxf(fabsf((float)tix), fabsf((float)tiy));
            unsigned flag = __ballot_sync(0xffffffffu, my_d >= 0 && sabs > kRefineKappa * tmax);
            while (flag) {
                const int e = __ffs(flag) - 1;
                flag &= flag - 1;
                // the subpixel point in FP64 from the staged position
                const double2 xy = make_double2(__shfl_sync(0xffffffffu, my_xy.x, e),
                                                __shfl_sync(0xffffffffu, my_xy.y, e));
                const double2 ti = qad_refine<R>(im.src, im.pitch, im.H, im.W, im.dtype == TOED_U8, sTab64,
                                                 2.0 * xy.x + 1.0, 2.0 * xy.y + 1.0, lane);
                if (lane == e) {
                    tix = ti.x;
                    tiy = ti.y;
                }
            }
            ori = (tix == 0.0 && tiy == 0.0) ? __int_as_float(0x7fc00000) : atan2f((float)tix, (float)(-tiy));
        } else {
            const float tix = gx * (2.f * fxx * fxx + 2.f * fxy * fxy) + gy * (2.f * fxx * fxy + 2.f * fyy * fxy) +
                              2.f * gx * gy * fxxy + gy * gy * fxyy + gx * gx * fxxx;
            const float tiy = gx * (2.f * fxx * fxy + 2.f * fyy * fxy) + gy * (2.f * fyy * fyy + 2.f * fxy * fxy) +
                              2.f * gx * gy * fxyy + gx * gx * fxxy + gy * gy * fyyy;
            ori = (tix == 0.f && tiy == 0.f) ? __int_as_float(0x7fc00000) : atan2f(tix, -tiy);
        }
        if (my_d < 0) continue;
        if (p.out_f64) {
            double2* o = reinterpret_cast<double2*>(im.out) + 2 * my_d;
            o[0] = my_xy;
            o[1] = make_double2((double)ori, (double)my_st.w);
        } else {
            reinterpret_cast<float4*>(im.out)[my_d] = make_float4((float)my_xy.x, (float)my_xy.y, ori, my_st.w);
        }
        if (im.index) im.index[my_d] = my_gi;
    }
}

static const void* scatter_qad_fn(int radius)
{
    const void* f = nullptr;
    switch (radius) {
    case 1: f = (const void*)fin_scatter_qad<1>; break;
    case 2: f = (const void*)fin_scatter_qad<2>; break;
    case 3: f = (const void*)fin_scatter_qad<3>; break;
    case 4: f = (const void*)fin_scatter_qad<4>; break;
    case 5: f = (const void*)fin_scatter_qad<5>; break;
    case 6: f = (const void*)fin_scatter_qad<6>; break;
    case 7: f = (const void*)fin_scatter_qad<7>; break;
    case 8: f = (const void*)fin_scatter_qad<8>; break;
    case 9: f = (const void*)fin_scatter_qad<9>; break;
    case 10: f = (const void*)fin_scatter_qad<10>; break;
    case 11: f = (const void*)fin_scatter_qad<11>; break;
    case 12: f = (const void*)fin_scatter_qad<12>; break;
    default: break;
    }
    return f;
}

cudaError_t preload_scatter_qad(int radius)
{
    const void* f = scatter_qad_fn(radius);
    if (!f) return cudaErrorInvalidValue;
    cudaFuncAttributes fa;
    return cudaFuncGetAttributes(&fa, f);
}

cudaError_t launch_scatter_qad(const BatchParams& p, cudaStream_t stream)
{
    const void* f = scatter_qad_fn(p.radius);
    if (!f) return cudaErrorInvalidValue;
    void* args[] = {const_cast<BatchParams*>(&p)};
    return cudaLaunchKernel(f, dim3(p.n_tiles), dim3(kQadThreads), args, 0, stream);
}

}  // namespace toed
