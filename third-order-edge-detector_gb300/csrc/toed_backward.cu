// toed_backward.cu -- adjoint of the fused detection with the selection
// frozen: gradients of every edgel's [x, y, orientation, strength] with
// respect to the image pixels and sigma.  The reference has no backward; the
// forward whose adjoint this is follows cpu_toed.cpp:128-545.
//
// One kernel, bw_adjoint<R>, in three phases per round of up to 32 edgels
// of a warp (every warp owns an equal run of edgels, sized so that the
// launch is one wave):
//   1. a warp per edgel re-evaluates, from the image, the nine derivatives
//      at the edgel's 2x-grid point P and Ix, Iy at the four NMS neighbours
//      of its (frozen) sector, each with its d/dsigma (one pass over the
//      union window of the five points, coalesced rows);
//   2. a thread per edgel runs the chain rule through the peak fit and the
//      third-order orientation (the peak fit's sums and the vector in FP64) and
//      accumulates dL/dsigma;
//   3. a warp per edgel adds the separable cotangent windows
//      sum_f X_f(q) V_f(p) of its five points onto the pixel gradient with
//      vector float reductions in global memory (cleared first by bw_clear,
//      one launch for the whole batch).
// Reductions from different edgels land in an unspecified order, so the
// pixel gradient is reproducible to float rounding, not bit for bit.
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>

#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

constexpr int kBwAdjThreads = 128;

struct BwImage {
    const void* src;
    long long pitch;
    const int* gidx;
    const void* gout;
    float* gpix;
    int H, W, dtype, n;
    int edgel_base;
};

struct BwParams {
    float tap[16][kMaxTaps];  // 0..3 G Gx Gxx Gxxx, 4..7 shifted by 1/2, 8..15 their d/dsigma
    int r;
    int out_f64;
    int n_img;
    int n_edgels;
    int per_warp;  // edgels per warp: all warps of the launch resident at once
    double* gsig;
    BwImage img[kBatchMax];
};

__device__ __forceinline__ void variants(int rho, int kap, int* xv, int* yv)
{
    const int a = rho & 1, b = kap & 1;
    *xv = (a == 0 && b == 0) ? 0 : (b ? 2 : 1);
    *yv = (a == 0 && b == 0) ? 0 : (a ? 2 : 1);
}

__device__ __forceinline__ float pix(const BwImage& im, int y, int x)
{
    if ((unsigned)y >= (unsigned)im.H || (unsigned)x >= (unsigned)im.W) return 0.f;
    const long long o = (long long)y * im.pitch + x;
    return im.dtype == TOED_U8 ? (float)__ldg((const unsigned char*)im.src + o) : __ldg((const float*)im.src + o);
}

// Tap tables with two zero entries on each side: entry k + 2 holds tap k, so
// a window offset by -1..+1 pixel (the NMS neighbours) indexes them without
// bounds tests.
template <int R>
__device__ __forceinline__ void build_tables_padded(const BwParams& p, float4* sA, float4* sS)
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4;
    for (int i = threadIdx.x; i < 3 * NTP; i += blockDim.x) {
        const int v = i / NTP, k = i - v * NTP - 2;
        const int f = (v == 2) ? 4 : 0;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), s = a;
        if (k >= 0 && k < NT && !(v == 0 && (k == 0 || k == NT - 1))) {
            a = make_float4(p.tap[f][k], p.tap[f + 1][k], p.tap[f + 2][k], p.tap[f + 3][k]);
            s = make_float4(p.tap[8 + f][k], p.tap[9 + f][k], p.tap[10 + f][k], p.tap[11 + f][k]);
        }
        sA[i] = a;
        sS[i] = s;
    }
}

// Per edgel, the 34 values the chain rule needs: the nine derivatives at P
// and their d/dsigma (0..17), then fx, fy, dfx/dsigma, dfy/dsigma at the four
// NMS neighbours A+, D+, A-, D- (18..33); slot 34 holds the sector bits.
constexpr int kNVal = 34;
constexpr int kValsPad = 37;  // row stride in shared memory (odd: conflict-free per-thread rows)
constexpr int kRedPad = 33;

// Sum over the union columns of value k (lane k): red[k][0..n) in a fixed order.
__device__ __forceinline__ float column_sum(const float* red_k, int n)
{
    float a = 0.f, b = 0.f;
    int t = 0;
    for (; t + 1 < n; t += 2) {
        a += red_k[t];
        b += red_k[t + 1];
    }
    if (t < n) a += red_k[t];
    return a + b;
}

// The 34 values of one edgel, evaluated by a whole warp as the reference
// defines the derivatives (cpu_toed.cpp:204-344): f = sum_{p,q} I(i-p, j-q)
// X(q) Y(p).  All five points' windows lie in the (NT+2) x (NT+2) union
// window around the edgel's pixel (i, j); lane c holds union column
// j-R-2+c, loads the union rows once (coalesced), contracts them with each
// point's y taps (lane-local), multiplies by its x taps, and the partial
// products are summed per value through shared memory.  The neighbours
// depend on the sector of P's (fx, fy), so P is summed first.  Lane 0's
// results land in row[0..33], the sector bits in row[34].
template <int R>
__device__ __forceinline__ void eval_edgel_warp(const BwImage& im, int rho, int kap, int lane, const float4* sA,
                                                const float4* sS, float (*red)[kRedPad], float* row)
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4, NU = NT + 2;
    const int i = rho >> 1, j = kap >> 1;
    const int col = j - R - 2 + lane;
    const bool okc = lane < NU && col >= 0 && col < im.W;
    float v[NU];
    if (im.dtype == TOED_U8) {
        const unsigned char* src = (const unsigned char*)im.src + col;
#pragma unroll
        for (int u = 0; u < NU; ++u) {
            const int y = i - R - 2 + u;
            v[u] = (okc && (unsigned)y < (unsigned)im.H) ? (float)__ldg(src + (long long)y * im.pitch) : 0.f;
        }
    } else {
        const float* src = (const float*)im.src + col;
#pragma unroll
        for (int u = 0; u < NU; ++u) {
            const int y = i - R - 2 + u;
            v[u] = (okc && (unsigned)y < (unsigned)im.H) ? __ldg(src + (long long)y * im.pitch) : 0.f;
        }
    }
    // ---- P: nine derivatives and their d/dsigma ----
    float pc0, pc1, ps0, ps1;  // P's (G, Gy) y contractions and their d/dsigma, for the neighbours
    int pyv;
    {
        int xv, yv;
        variants(rho, kap, &xv, &yv);
        pyv = yv;
        // y tap of union row u: pp = NT - u (entry NT + 2 - u); x tap of lane: qq = NT - lane
        const float4* YA = sA + yv * NTP + NT + 2;
        const float4* YS = sS + yv * NTP + NT + 2;
        float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
        for (int u = 0; u < NU; ++u) {
            const float4 ya = YA[-u], ys = YS[-u];
            c0 = fmaf(v[u], ya.x, c0); c1 = fmaf(v[u], ya.y, c1);
            c2 = fmaf(v[u], ya.z, c2); c3 = fmaf(v[u], ya.w, c3);
            s0 = fmaf(v[u], ys.x, s0); s1 = fmaf(v[u], ys.y, s1);
            s2 = fmaf(v[u], ys.z, s2); s3 = fmaf(v[u], ys.w, s3);
        }
        if (lane < NU) {
            const float4 xa = sA[xv * NTP + NT + 2 - lane], xs = sS[xv * NTP + NT + 2 - lane];
            // fx (Gx,G) fy (G,Gy) fxx (Gxx,G) fxy (Gx,Gy) fyy (G,Gyy)
            // fxxy (Gxx,Gy) fxyy (Gx,Gyy) fxxx (Gxxx,G) fyyy (G,Gyyy)
            red[0][lane] = xa.y * c0;  red[9][lane] = fmaf(xs.y, c0, xa.y * s0);
            red[1][lane] = xa.x * c1;  red[10][lane] = fmaf(xs.x, c1, xa.x * s1);
            red[2][lane] = xa.z * c0;  red[11][lane] = fmaf(xs.z, c0, xa.z * s0);
            red[3][lane] = xa.y * c1;  red[12][lane] = fmaf(xs.y, c1, xa.y * s1);
            red[4][lane] = xa.x * c2;  red[13][lane] = fmaf(xs.x, c2, xa.x * s2);
            red[5][lane] = xa.z * c1;  red[14][lane] = fmaf(xs.z, c1, xa.z * s1);
            red[6][lane] = xa.y * c2;  red[15][lane] = fmaf(xs.y, c2, xa.y * s2);
            red[7][lane] = xa.w * c0;  red[16][lane] = fmaf(xs.w, c0, xa.w * s0);
            red[8][lane] = xa.x * c3;  red[17][lane] = fmaf(xs.x, c3, xa.x * s3);
        }
        __syncwarp();
        if (lane < 18) row[lane] = column_sum(red[lane], NU);
        __syncwarp();
        pc0 = c0; pc1 = c1; ps0 = s0; ps1 = s1;
    }
    // ---- the frozen sector (cpu_toed.cpp:415-462 in closed form) and the
    // four neighbours' fx, fy with their d/dsigma ----
    const float fx = row[0], fy = row[1];
    const bool xmaj = fabsf(fx) >= fabsf(fy);
    const int sx = fx >= 0.f ? 1 : -1, sy = fy >= 0.f ? 1 : -1;
    const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
    const int nr[4] = {rho + ar, rho + sy, rho - ar, rho - sy};  // A+, D+, A-, D-
    const int nc[4] = {kap + ac, kap + sx, kap - ac, kap - sx};
    // A point's y contractions depend only on its y taps (variant yv) and
    // its row offset di: a neighbour that shares both with P or with an
    // earlier neighbour (in x-major sectors A+ and A- always do, and both
    // share P's when P is on an odd 2x row) reuses those sums -- the same
    // products in the same order, so the values are identical.
    float qcg[4], qcy[4], qsg[4], qsy[4];
    int qkey[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int xv, yv;
        variants(nr[q], nc[q], &xv, &yv);
        const int di = (nr[q] >> 1) - i, dj = (nc[q] >> 1) - j;
        const int key = yv * 4 + (di + 1);
        qkey[q] = key;
        float cg = 0.f, cy = 0.f, sg = 0.f, sy_ = 0.f;
        int from = -1;  // an earlier neighbour with the same sums (warp-uniform)
#pragma unroll
        for (int q2 = 0; q2 < q; ++q2)
            if (from < 0 && qkey[q2] == key) from = q2;
        if (key == pyv * 4 + 1) {
            cg = pc0; cy = pc1; sg = ps0; sy_ = ps1;
        } else if (from >= 0) {
#pragma unroll
            for (int q2 = 0; q2 < q; ++q2)
                if (q2 == from) { cg = qcg[q2]; cy = qcy[q2]; sg = qsg[q2]; sy_ = qsy[q2]; }
        } else {
            const float4* YA = sA + yv * NTP + NT + 2 + di;
            const float4* YS = sS + yv * NTP + NT + 2 + di;
#pragma unroll
            for (int u = 0; u < NU; ++u) {
                const float4 ya = YA[-u], ys = YS[-u];
                cg = fmaf(v[u], ya.x, cg); cy = fmaf(v[u], ya.y, cy);
                sg = fmaf(v[u], ys.x, sg); sy_ = fmaf(v[u], ys.y, sy_);
            }
        }
        qcg[q] = cg; qcy[q] = cy; qsg[q] = sg; qsy[q] = sy_;
        if (lane < NU) {
            const float4 xa = sA[xv * NTP + NT + 2 + dj - lane], xs = sS[xv * NTP + NT + 2 + dj - lane];
            red[18 + 4 * q][lane] = xa.y * cg;                   // fx (Gx, G)
            red[19 + 4 * q][lane] = xa.x * cy;                   // fy (G, Gy)
            red[20 + 4 * q][lane] = fmaf(xs.y, cg, xa.y * sg);   // d/dsigma
            red[21 + 4 * q][lane] = fmaf(xs.x, cy, xa.x * sy_);
        }
    }
    __syncwarp();
    if (lane < 16) row[18 + lane] = column_sum(red[18 + lane], NU);
    if (lane == 0) row[34] = __int_as_float((xmaj ? 1 : 0) | (sx > 0 ? 2 : 0) | (sy > 0 ? 4 : 0));
    __syncwarp();
}

constexpr int kBwV = 12;  // y-vectors per union row: P's four, two per neighbour

// Scatter of one edgel's cotangents onto the pixel gradient, by a whole
// warp: grad I(u) += sum over the five points and their filters of
// X_f(q) V_f(p), V_f = the y taps weighted by the point's cotangents.  All
// five windows lie in the (NT+2) x (NT+2) union window around the edgel's
// pixel; lane c takes union column c and holds the x taps of the five points
// there (12 values), lane r first stages the y-vectors of union row r in
// shared memory, then each union row is added with one vector reduction
// (red.global.add.f32) per lane.  The grid pixels outside the image are the
// zero padding and receive nothing.
template <int R>
__device__ __forceinline__ void scatter_edgel_warp(const BwImage& im, int rho, int kap, int lane, const float4* sA,
                                                   const float* g, float4 (*sV)[kBwV / 4])
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4, NU = NT + 2;
    const int bits = __float_as_int(g[17]);
    const bool xmaj = bits & 1;
    const int sx = (bits & 2) ? 1 : -1, sy = (bits & 4) ? 1 : -1;
    const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
    const int pr[5] = {rho, rho + ar, rho + sy, rho - ar, rho - sy};  // P, A+, D+, A-, D-
    const int pc[5] = {kap, kap + ac, kap + sx, kap - ac, kap - sx};
    const int i = rho >> 1, j = kap >> 1;
    float4 xP = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 xN[4];
    float4 v0 = make_float4(0.f, 0.f, 0.f, 0.f), v1 = v0, v2 = v0;
    const int l = lane < NU ? lane : NU - 1;  // lanes past the window repeat the last column (unused)
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        int xv, yv;
        variants(pr[q], pc[q], &xv, &yv);
        const int di = (pr[q] >> 1) - i, dj = (pc[q] >> 1) - j;
        // padded entries: x tap of union column l = NT + 2 + dj - l, y tap of union row l = NT + 2 + di - l
        const float4 x = sA[xv * NTP + NT + 2 + dj - l];
        const float4 y = sA[yv * NTP + NT + 2 + di - l];
        if (q == 0) {
            xP = x;
            v0.x = g[1] * y.y + g[4] * y.z + g[8] * y.w;  // G    x (fy, fyy, fyyy)
            v0.y = g[0] * y.x + g[3] * y.y + g[6] * y.z;  // Gx   x (fx, fxy, fxyy)
            v0.z = g[2] * y.x + g[5] * y.y;               // Gxx  x (fxx, fxxy)
            v0.w = g[7] * y.x;                            // Gxxx x fxxx
        } else {
            xN[q - 1] = make_float2(x.x, x.y);
            const float a = g[8 + 2 * q] * y.y, b = g[7 + 2 * q] * y.x;  // G x fy, Gx x fx at the neighbour
            if (q == 1) { v1.x = a; v1.y = b; }
            else if (q == 2) { v1.z = a; v1.w = b; }
            else if (q == 3) { v2.x = a; v2.y = b; }
            else { v2.z = a; v2.w = b; }
        }
    }
    if (lane < NU) {
        sV[lane][0] = v0;
        sV[lane][1] = v1;
        sV[lane][2] = v2;
    }
    __syncwarp();
    const int x = j - R - 2 + lane;
    const bool okx = lane < NU && x >= 0 && x < im.W;
    float* out = im.gpix + x;
    for (int r = 0; r < NU; ++r) {
        const int y = i - R - 2 + r;
        const float4 a = sV[r][0], b = sV[r][1], c = sV[r][2];
        float v = xP.x * a.x;
        v = fmaf(xP.y, a.y, v);
        v = fmaf(xP.z, a.z, v);
        v = fmaf(xP.w, a.w, v);
        v = fmaf(xN[0].x, b.x, v);
        v = fmaf(xN[0].y, b.y, v);
        v = fmaf(xN[1].x, b.z, v);
        v = fmaf(xN[1].y, b.w, v);
        v = fmaf(xN[2].x, c.x, v);
        v = fmaf(xN[2].y, c.y, v);
        v = fmaf(xN[3].x, c.z, v);
        v = fmaf(xN[3].y, c.w, v);
        if (okx && (unsigned)y < (unsigned)im.H) atomicAdd(out + (long long)y * im.W, v);
    }
    __syncwarp();
}

// bw_adjoint: every warp owns p.per_warp consecutive edgels (the host sizes
// the run so that all warps of the launch are resident at once: no second,
// nearly empty wave) and takes them in rounds of up to 32.  Phase 1: the
// warp evaluates the round's edgels one after another (eval_edgel_warp).
// Phase 2: one lane per edgel runs the chain rule.  The peak fit's
// cancellations (fp - fm, fp + fm - 2f) and the third-order vector
// (TIx, TIy) are formed in FP64, as in the forward; the rest is FP32.
// Phase 3: the warp scatters the round's cotangents onto the pixel
// gradient (scatter_edgel_warp), which the host cleared beforehand.  The
// phases exchange data only within the warp.
template <int R>
__global__ void __launch_bounds__(kBwAdjThreads) bw_adjoint(const __grid_constant__ BwParams p)
{
    constexpr int NT = 2 * R + 3, NTP = NT + 4;
    __shared__ float4 sA[3 * NTP], sS[3 * NTP];
    __shared__ float sVal[kBwAdjThreads][kValsPad];
    __shared__ float sRed[kBwAdjThreads / 32][kNVal][kRedPad];
    __shared__ float4 sV[kBwAdjThreads / 32][NT + 2][kBwV / 4];
    build_tables_padded<R>(p, sA, sS);
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long wfirst = ((long long)blockIdx.x * (kBwAdjThreads / 32) + wid) * p.per_warp;
    const int wend = (int)min((long long)p.n_edgels, wfirst + p.per_warp);
    double gsig = 0.0;
    for (int ebase = (int)min(wfirst, (long long)p.n_edgels); ebase < wend; ebase += 32) {
        const int nw = min(32, wend - ebase);
        const int e = ebase + lane;
        // each lane resolves its own edgel's image and 2x-grid point
        int my_k = 0, my_rho = 0, my_kap = 0;
        if (lane < nw) {
            my_k = find_image(p.n_img, e, [&](int i) { return p.img[i].edgel_base; });
            const BwImage& im = p.img[my_k];
            const int gi = im.gidx[e - im.edgel_base], W2 = 2 * im.W;
            my_rho = gi / W2;
            my_kap = gi - my_rho * W2;
        }
        // ---- phase 1: warp-cooperative evaluation, one edgel at a time ----
        for (int jj = 0; jj < nw; ++jj) {
            const int k = __shfl_sync(0xffffffffu, my_k, jj);
            const int rho = __shfl_sync(0xffffffffu, my_rho, jj), kap = __shfl_sync(0xffffffffu, my_kap, jj);
            eval_edgel_warp<R>(p.img[k], rho, kap, lane, sA, sS, sRed[wid], sVal[wid * 32 + jj]);
        }
        __syncwarp();
        // ---- phase 2: the chain rule, one thread per edgel ----
        if (lane < nw) {
            const BwImage& im = p.img[my_k];
            const int local = e - im.edgel_base;
            const float* row = sVal[threadIdx.x];
            float go[4];
            if (p.out_f64) {
                const double* g = (const double*)im.gout + 4LL * local;
                go[0] = (float)g[0]; go[1] = (float)g[1]; go[2] = (float)g[2]; go[3] = (float)g[3];
            } else {
                const float* g = (const float*)im.gout + 4LL * local;
                go[0] = g[0]; go[1] = g[1]; go[2] = g[2]; go[3] = g[3];
            }
            const int bits = __float_as_int(row[34]);
            const bool xmaj = bits & 1;
            const int sx = (bits & 2) ? 1 : -1, sy = (bits & 4) ? 1 : -1;
            const float fx = row[0], fy = row[1], fxx = row[2], fxy = row[3], fyy = row[4], fxxy = row[5],
                        fxyy = row[6], fxxx = row[7], fyyy = row[8];
            float nd[4][2], M[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                nd[q][0] = row[18 + 4 * q];
                nd[q][1] = row[19 + 4 * q];
                M[q] = sqrtf(nd[q][0] * nd[q][0] + nd[q][1] * nd[q][1]);
            }
            // ---- forward values ----
            const float m = sqrtf(fx * fx + fy * fy);
            const float rm = 1.f / m;
            const float nx = fx * rm, ny = fy * rm;
            const float c = (float)(sx * sy);
            const float t = xmaj ? c * fy / fx : c * fx / fy;  // slope |ny|/|nx| or |nx|/|ny|
            float num, den;
            {
                const double td = t;
                const double fp = (double)M[0] * (1.0 - td) + (double)M[1] * td;
                const double fm = (double)M[2] * (1.0 - td) + (double)M[3] * td;
                num = (float)(fp - fm);
                den = (float)(fm + fp - 2.0 * (double)m);
            }
            const float rden = 1.f / den;
            const float S = sqrtf(1.f + t * t);
            const float sst = -0.5f * num * S * rden;
            // ---- reverse: position, strength ----
            const float g_sst = 0.5f * (go[0] * nx + go[1] * ny);
            const float g_nx = 0.5f * go[0] * sst, g_ny = 0.5f * go[1] * sst;
            const float g_maxf = go[3];  // strength = |max_f| |n| = max_f (max_f > 0 at a maximum)
            const float g_num = -0.5f * S * rden * g_sst - 0.25f * num * rden * g_maxf;
            const float g_den = 0.5f * num * S * rden * rden * g_sst + 0.125f * num * num * rden * rden * g_maxf;
            float g_t = g_sst * (-0.5f * num * rden) * t / S;
            const float g_m = g_maxf - 2.f * g_den;
            const float g_fp = g_num + g_den, g_fm = -g_num + g_den;
            const float gM[4] = {g_fp * (1.f - t), g_fp * t, g_fm * (1.f - t), g_fm * t};
            g_t += g_fp * (M[1] - M[0]) + g_fm * (M[3] - M[2]);
            float gfx = 0.f, gfy = 0.f;
            if (xmaj) {
                gfx += g_t * (-t / fx);
                gfy += g_t * (c / fx);
            } else {
                gfx += g_t * (c / fy);
                gfy += g_t * (-t / fy);
            }
            const float rm3 = rm * rm * rm;
            gfx += g_nx * (rm - fx * fx * rm3) + g_ny * (-fx * fy * rm3) + g_m * fx * rm;
            gfy += g_nx * (-fx * fy * rm3) + g_ny * (rm - fy * fy * rm3) + g_m * fy * rm;
            // ---- reverse: orientation atan2(TIx, -TIy) (cpu_toed.cpp:227-232) ----
            float gP[9];
            gP[2] = gP[3] = gP[4] = gP[5] = gP[6] = gP[7] = gP[8] = 0.f;
            if (go[2] != 0.f) {
                const double dx = fx, dy = fy, dxx = fxx, dxy = fxy, dyy = fyy;
                const double TIx = dx * (2 * dxx * dxx + 2 * dxy * dxy) + dy * (2 * dxx * dxy + 2 * dyy * dxy) +
                                   2 * dx * dy * (double)fxxy + dy * dy * (double)fxyy + dx * dx * (double)fxxx;
                const double TIy = dx * (2 * dxx * dxy + 2 * dyy * dxy) + dy * (2 * dyy * dyy + 2 * dxy * dxy) +
                                   2 * dx * dy * (double)fxyy + dx * dx * (double)fxxy + dy * dy * (double)fyyy;
                const float tix = (float)TIx, tiy = (float)TIy;
                const float q2 = tix * tix + tiy * tiy;
                if (q2 > 0.f) {
                    const float gX = go[2] * (-tiy) / q2, gY = go[2] * tix / q2;
                    gfx += gX * (2 * fxx * fxx + 2 * fxy * fxy + 2 * fy * fxxy + 2 * fx * fxxx) +
                           gY * (2 * fxx * fxy + 2 * fyy * fxy + 2 * fy * fxyy + 2 * fx * fxxy);
                    gfy += gX * (2 * fxx * fxy + 2 * fyy * fxy + 2 * fx * fxxy + 2 * fy * fxyy) +
                           gY * (2 * fyy * fyy + 2 * fxy * fxy + 2 * fx * fxyy + 2 * fy * fyyy);
                    gP[2] = gX * (4 * fx * fxx + 2 * fy * fxy) + gY * (2 * fx * fxy);
                    gP[3] = gX * (4 * fx * fxy + 2 * fy * fxx + 2 * fy * fyy) + gY * (2 * fx * fxx + 2 * fx * fyy + 4 * fy * fxy);
                    gP[4] = gX * (2 * fy * fxy) + gY * (2 * fx * fxy + 4 * fy * fyy);
                    gP[5] = gX * (2 * fx * fy) + gY * (fx * fx);
                    gP[6] = gX * (fy * fy) + gY * (2 * fx * fy);
                    gP[7] = gX * (fx * fx);
                    gP[8] = gY * (fy * fy);
                }
            }
            gP[0] = gfx;
            gP[1] = gfy;
            // the cotangents replace the values in this thread's own row:
            // [0..8] at P, [9 + 2q, 10 + 2q] = (gx, gy) at neighbour q, [17] sector
            float* rec = sVal[threadIdx.x];
            float gs = 0.f;
#pragma unroll
            for (int q = 0; q < 9; ++q) gs = fmaf(gP[q], row[9 + q], gs);
            float gN[8];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float rM = gM[q] / M[q];
                gN[2 * q] = rM * nd[q][0];
                gN[2 * q + 1] = rM * nd[q][1];
                gs = fmaf(gN[2 * q], row[20 + 4 * q], fmaf(gN[2 * q + 1], row[21 + 4 * q], gs));
            }
            const float sec = row[34];
#pragma unroll
            for (int q = 0; q < 9; ++q) rec[q] = gP[q];
#pragma unroll
            for (int q = 0; q < 8; ++q) rec[9 + q] = gN[q];
            rec[17] = sec;
            gsig += gs;
        }
        __syncwarp();
        // ---- phase 3: scatter, a warp per edgel (scatter_edgel_warp) ----
        for (int jj = 0; jj < nw; ++jj) {
            const int k = __shfl_sync(0xffffffffu, my_k, jj);
            const int rho = __shfl_sync(0xffffffffu, my_rho, jj), kap = __shfl_sync(0xffffffffu, my_kap, jj);
            scatter_edgel_warp<R>(p.img[k], rho, kap, lane, sA, sVal[wid * 32 + jj], sV[wid]);
        }
        __syncwarp();  // the next round rewrites this warp's rows
    }
    // dL/dsigma: warp sums in FP64, one FP64 atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gsig += __shfl_down_sync(0xffffffffu, gsig, o);
    if (lane == 0 && gsig != 0.0) atomicAdd(p.gsig, gsig);
}

// Resident CTAs of bw_adjoint<R> on each device (SMs x CTAs per SM), found once.
constexpr int kBwMaxDevices = 64;

template <int R>
static int bw_resident_ctas()
{
    static std::atomic<int> cache[kBwMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kBwMaxDevices) return 0;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n == 0) {
        int sms = 0, bps = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, bw_adjoint<R>, kBwAdjThreads, 0) != cudaSuccess)
            return 0;
        n = sms * bps;
        cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

template <int R>
static cudaError_t launch_bw(BwParams& p, cudaStream_t stream)
{
    if (p.n_edgels == 0) return cudaSuccess;
    // every warp the same run of edgels, as short as keeps the launch in one
    // wave (32 a warp if the occupancy is unknown)
    const long long warps = (long long)bw_resident_ctas<R>() * (kBwAdjThreads / 32);
    p.per_warp = warps > 0 ? (int)((p.n_edgels + warps - 1) / warps) : 32;
    const long long per_cta = (long long)p.per_warp * (kBwAdjThreads / 32);
    void* args[] = {&p};
    return cudaLaunchKernel((const void*)bw_adjoint<R>, dim3((unsigned)((p.n_edgels + per_cta - 1) / per_cta)),
                            dim3(kBwAdjThreads), args, 0, stream);
}

// Clears dL/dI of image blockIdx.y (rows of width W, contiguous): 16-byte
// stores from the first 16-byte boundary, scalar stores around them.
__global__ void __launch_bounds__(256) bw_clear(const __grid_constant__ BwParams p)
{
    const BwImage& d = p.img[blockIdx.y];
    float* g = d.gpix;
    const long long npx = (long long)d.H * d.W;
    const long long head = min(npx, (long long)(((16u - (reinterpret_cast<uintptr_t>(g) & 15u)) & 15u) / 4u));
    const long long nv = (npx - head) / 4;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
    float4* g4 = reinterpret_cast<float4*>(g + head);
    for (long long i = t0; i < nv; i += st) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (t0 < head) g[t0] = 0.f;
    const long long tail = head + 4 * nv;
    if (t0 < npx - tail) g[tail + t0] = 0.f;
}

cudaError_t backward_launch(const toed_grad_image* items, int n, const toed_params* prm, int r, double* gsig,
                            cudaStream_t stream)
{
    std::unique_ptr<BwParams> pp(new BwParams());
    BwParams& p = *pp;
    std::memset(&p, 0, sizeof(p));
    const double s = prm->sigma, nrm = std::sqrt(2.0 * 3.14159265358979323846);
    for (int sh = 0; sh < 2; ++sh)
        for (int k = 0; k < 2 * r + 3; ++k) {
            const double x = (double)(k - (r + 1)) + (sh ? 0.5 : 0.0);
            const double e = std::exp(-(x * x) / (2.0 * s * s));
            const double G = e / (nrm * s), Gx = (-x * e) / (nrm * s * s * s);
            const double Gxx = ((x * x - s * s) * e) / (nrm * s * s * s * s * s);
            const double Gxxx = ((x * (3.0 * s * s - x * x)) * e) / (nrm * s * s * s * s * s * s * s);
            const double q = x * x / (s * s * s);  // d e / d sigma = e * x^2 / sigma^3
            const double v[8] = {G, Gx, Gxx, Gxxx, G * (q - 1.0 / s), Gx * (q - 3.0 / s),
                                 -2.0 * s * e / (nrm * s * s * s * s * s) + Gxx * (q - 5.0 / s),
                                 6.0 * s * x * e / (nrm * s * s * s * s * s * s * s) + Gxxx * (q - 7.0 / s)};
            for (int f = 0; f < 4; ++f) {
                p.tap[4 * sh + f][k] = (float)v[f];
                p.tap[8 + 4 * sh + f][k] = (float)v[4 + f];
            }
        }
    p.r = r;
    p.out_f64 = prm->out_dtype == TOED_F64;
    p.n_img = n;
    p.gsig = gsig;
    int edg = 0;
    for (int i = 0; i < n; ++i) {
        BwImage& d = p.img[i];
        d.src = items[i].pixels;
        d.pitch = items[i].pitch;
        d.gidx = items[i].grid_index;
        d.gout = items[i].grad_edgels;
        d.gpix = items[i].grad_pixels;
        d.H = items[i].height;
        d.W = items[i].width;
        d.dtype = items[i].dtype;
        d.n = items[i].n_edgels;
        d.edgel_base = edg;
        edg += d.n;
    }
    p.n_edgels = edg;
    {
        // dL/dI of every image cleared by one launch (the scatter adds into it)
        void* args[] = {&p};
        const cudaError_t e = cudaLaunchKernel((const void*)bw_clear, dim3(64, n), dim3(256), args, 0, stream);
        if (e != cudaSuccess) return e;
    }
    switch (r) {
    case 1: return launch_bw<1>(p, stream);
    case 2: return launch_bw<2>(p, stream);
    case 3: return launch_bw<3>(p, stream);
    case 4: return launch_bw<4>(p, stream);
    case 5: return launch_bw<5>(p, stream);
    case 6: return launch_bw<6>(p, stream);
    case 7: return launch_bw<7>(p, stream);
    case 8: return launch_bw<8>(p, stream);
    case 9: return launch_bw<9>(p, stream);
    case 10: return launch_bw<10>(p, stream);
    case 11: return launch_bw<11>(p, stream);
    case 12: return launch_bw<12>(p, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace toed
