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
//      32 records lane e forms record e's third-order vector (FP64 in HYBRID
//      precision, all lanes busy), the angle and the output record.
#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

namespace {

constexpr int kQadThreads = 128;
constexpr int kQadSegPerThread = kSegTile / kQadThreads;

// Keys cubic convolution kernel, a = -1/2 (subpix_to_correction.cpp:57-67).
__device__ __forceinline__ float keys(float s)
{
    const float a = -0.5f, x = fabsf(s);
    if (x <= 1.f) return ((a + 2.f) * x - (a + 3.f)) * x * x + 1.f;
    if (x < 2.f) return ((a * x - 5.f * a) * x + 8.f * a) * x - 4.f * a;
    return 0.f;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

}  // namespace

// The nine derivatives of one (x taps, y contraction) pairing, added in:
// x = (G, Gx, Gxx, Gxxx) taps of this lane's column (weighted), c = the
// column's contractions with (G, Gy, Gyy, Gyyy).
__device__ __forceinline__ void qad_pair(float4 x, float4 c, float (&acc)[9])
{
    acc[0] = fmaf(x.y, c.x, acc[0]);  // fx   = Gx   (x) G
    acc[1] = fmaf(x.x, c.y, acc[1]);  // fy   = G    (x) Gy
    acc[2] = fmaf(x.z, c.x, acc[2]);  // fxx  = Gxx  (x) G
    acc[3] = fmaf(x.y, c.y, acc[3]);  // fxy  = Gx   (x) Gy
    acc[4] = fmaf(x.x, c.z, acc[4]);  // fyy  = G    (x) Gyy
    acc[5] = fmaf(x.z, c.y, acc[5]);  // fxxy = Gxx  (x) Gy
    acc[6] = fmaf(x.y, c.z, acc[6]);  // fxyy = Gx   (x) Gyy
    acc[7] = fmaf(x.w, c.x, acc[7]);  // fxxx = Gxxx (x) G
    acc[8] = fmaf(x.x, c.w, acc[8]);  // fyyy = G    (x) Gyyy
}

__device__ __forceinline__ float4 f4_fma(float a, float4 x, float4 y)
{
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}

__device__ __forceinline__ float4 f4_scale(float a, float4 x) { return make_float4(a * x.x, a * x.y, a * x.z, a * x.w); }

// Interpolation is linear, so the four columns of the 4 x 4 block fold into
// three weighted x-tap vectors per lane, one per x variant in use: columns
// of parity b = 0 take T taps in rows of parity a = 0 and F taps in rows
// a = 1; columns b = 1 take S taps.  The columns' parities alternate from
// X1 - 1, so B0 (0 or 1) is the parity of the block's first column.
template <int R, int B0>
__device__ __forceinline__ void qad_columns(const float4* __restrict__ sTab, int X1, int j, int l,
                                            const float (&wx)[4], float4& xT, float4& xF, float4& xS)
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4;
    xT = xF = xS = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int dj = ((X1 - 1 + s) >> 1) - j;
        const int e = NT + 2 + dj - l;  // padded entry of this lane's column
        if (((B0 + s) & 1) == 0) {
            xT = f4_fma(wx[s], sTab[e], xT);
            xF = f4_fma(wx[s], sTab[NTP + e], xF);
        } else {
            xS = f4_fma(wx[s], sTab[2 * NTP + e], xS);
        }
    }
}

// One row of the 4 x 4 block: 2x-grid row parity A, original row offset DI
// from the window centre (both fixed by the parity of the block's first row).
// Contracts this lane's window column with the row's y taps -- shifted (S)
// for A = 1; full (F) for A = 0, the truncated set (T) being F without its
// two end taps -- weights it by the row's Keys weight and adds the row's
// sub-grids: (0,0) T x T, (0,1) S x F, (1,0) F x S, (1,1) S x S (x by y).
template <int R, int A, int DI>
__device__ __forceinline__ void qad_row(const float (&v)[2 * R + 5], const float4* __restrict__ sTab, float wy,
                                        float4 xT, float4 xF, float4 xS, float (&acc)[9])
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4, NU = NT + 2;
    const float4* Yt = sTab + (A ? 2 : 1) * NTP + NT + 2 + DI;  // entry NT + 2 + DI - u: tap of window row u
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < NU; ++u) {
        const float4 y = Yt[-u];
        c.x = fmaf(v[u], y.x, c.x); c.y = fmaf(v[u], y.y, c.y);
        c.z = fmaf(v[u], y.z, c.z); c.w = fmaf(v[u], y.w, c.w);
    }
    if (A) {
        const float4 cs = f4_scale(wy, c);
        qad_pair(xF, cs, acc);
        qad_pair(xS, cs, acc);
    } else {
        // T = F less the taps k = 0 (window row NT + DI) and k = NT - 1 (window row DI + 1)
        const float4 e0 = sTab[NTP + 2], e1 = sTab[NTP + 2 + NT - 1];
        const float va = v[NT + DI], vb = v[DI + 1];
        float4 t;
        t.x = fmaf(-vb, e1.x, fmaf(-va, e0.x, c.x));
        t.y = fmaf(-vb, e1.y, fmaf(-va, e0.y, c.y));
        t.z = fmaf(-vb, e1.z, fmaf(-va, e0.z, c.z));
        t.w = fmaf(-vb, e1.w, fmaf(-va, e0.w, c.w));
        qad_pair(xT, f4_scale(wy, t), acc);
        qad_pair(xS, f4_scale(wy, c), acc);
    }
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
    // per warp, the nine derivatives of the 32 records in flight (stride 9: conflict-free per lane)
    __shared__ float sDer[kQadThreads / 32][32 * 9];
    for (int i = threadIdx.x; i < 3 * NTP; i += kQadThreads) {
        const int v = i / NTP, k = i - v * NTP - 2;
        const int f = (v == 2) ? 4 : 0;
        float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
        if (k >= 0 && k < NT && !(v == 0 && (k == 0 || k == NT - 1)))
            t = make_float4(p.taps.v[f][k], p.taps.v[f + 1][k], p.taps.v[f + 2][k], p.taps.v[f + 3][k]);
        sTab[i] = t;
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
                const double2 xy = *reinterpret_cast<const double2*>(&p.sc.staging[src]);
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
            const int j = X1 >> 1;
            // 1. the Keys weights of the 4 x 4 block around the subpixel point
            float wx[4], wy[4];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                wx[s] = keys(tx + 1.f - (float)s);
                wy[s] = keys(ty + 1.f - (float)s);
            }
            // 3. the block's columns folded into three x-tap vectors, then its
            // four rows Y1 - 1 .. Y1 + 2 (parities and offsets follow Y1's parity)
            float4 xT, xF, xS;
            if ((X1 & 1) == 0)
                qad_columns<R, 1>(sTab, X1, j, l, wx, xT, xF, xS);
            else
                qad_columns<R, 0>(sTab, X1, j, l, wx, xT, xF, xS);
            float acc[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) acc[q] = 0.f;
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
        if (my_d < 0) continue;
        const double4_32a my_rc = p.sc.staging[my_src];
        // the third-order vector, the angle and the output record
        const float gx = mine[0], gy = mine[1], fxx = mine[2], fxy = mine[3], fyy = mine[4], fxxy = mine[5],
                    fxyy = mine[6], fxxx = mine[7], fyyy = mine[8];
        float ori;
        if (p.hyb) {
            const double dfx = gx, dfy = gy, dxx = fxx, dxy = fxy, dyy = fyy;
            const double tix = dfx * (2.0 * dxx * dxx + 2.0 * dxy * dxy) + dfy * (2.0 * dxx * dxy + 2.0 * dyy * dxy) +
                               2.0 * dfx * dfy * (double)fxxy + dfy * dfy * (double)fxyy + dfx * dfx * (double)fxxx;
            const double tiy = dfx * (2.0 * dxx * dxy + 2.0 * dyy * dxy) + dfy * (2.0 * dyy * dyy + 2.0 * dxy * dxy) +
                               2.0 * dfx * dfy * (double)fxyy + dfx * dfx * (double)fxxy + dfy * dfy * (double)fyyy;
            ori = (tix == 0.0 && tiy == 0.0) ? __int_as_float(0x7fc00000) : atan2f((float)tix, (float)(-tiy));
        } else {
            const float tix = gx * (2.f * fxx * fxx + 2.f * fxy * fxy) + gy * (2.f * fxx * fxy + 2.f * fyy * fxy) +
                              2.f * gx * gy * fxxy + gy * gy * fxyy + gx * gx * fxxx;
            const float tiy = gx * (2.f * fxx * fxy + 2.f * fyy * fxy) + gy * (2.f * fyy * fyy + 2.f * fxy * fxy) +
                              2.f * gx * gy * fxyy + gx * gx * fxxy + gy * gy * fyyy;
            ori = (tix == 0.f && tiy == 0.f) ? __int_as_float(0x7fc00000) : atan2f(tix, -tiy);
        }
        if (p.out_f64) {
            double2* o = reinterpret_cast<double2*>(im.out) + 2 * my_d;
            o[0] = make_double2(my_rc.x, my_rc.y);
            o[1] = make_double2((double)ori, my_rc.w);
        } else {
            reinterpret_cast<float4*>(im.out)[my_d] =
                make_float4((float)my_rc.x, (float)my_rc.y, ori, (float)my_rc.w);
        }
        if (im.index) im.index[my_d] = p.sc.staging_idx[my_src];
    }
}

cudaError_t launch_scatter_qad(const BatchParams& p, cudaStream_t stream)
{
    const void* f = nullptr;
    switch (p.radius) {
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
    default: return cudaErrorInvalidValue;
    }
    void* args[] = {const_cast<BatchParams*>(&p)};
    return cudaLaunchKernel(f, dim3(p.n_tiles), dim3(kQadThreads), args, 0, stream);
}

}  // namespace toed
