// toed_backward.cu -- adjoint of the fused detection with the selection
// frozen: gradients of every edgel's [x, y, orientation, strength] with
// respect to the image pixels and sigma.  The reference has no backward; the
// forward whose adjoint this is follows cpu_toed.cpp:128-545.
//
// bw_adjoint<R>  one thread per edgel: re-evaluates, from the image, the nine
//                derivatives at the edgel's 2x-grid point P and Ix, Iy at the
//                four NMS neighbours of its (frozen) sector, each with its
//                d/dsigma, then runs the chain rule through the peak fit and
//                the third-order orientation in FP64; writes 17 cotangents
//                per edgel and accumulates dL/dsigma.
// bw_scatter<R>  one CTA per 32x32 pixel tile: finds the edgels whose
//                windows reach the tile (binary search on the row-major grid
//                index), adds each point's separable cotangent window
//                sum_f X_f(q) V_f(p) into a shared-memory tile, writes the
//                tile -- no global atomics; every pixel written once.
#include <cmath>
#include <cstring>
#include <memory>

#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

constexpr int kBwT = 32;    // scatter tile side
constexpr int kCotW = 18;   // floats per edgel cotangent record (17 + sector bits)
constexpr int kBwAdjThreads = 128;

struct BwImage {
    const void* src;
    long long pitch;
    const int* gidx;
    const void* gout;
    float* gpix;
    int H, W, dtype, n;
    int edgel_base;
    int ntx, nty, tile_base;
};

struct BwParams {
    float tap[16][kMaxTaps];  // 0..3 G Gx Gxx Gxxx, 4..7 shifted by 1/2, 8..15 their d/dsigma
    int r;
    int out_f64;
    int n_img;
    int n_edgels;
    int n_tiles;
    float* cot;               // n_edgels x kCotW
    double* gsig;
    BwImage img[kBatchMax];
};

// Shared tap tables per variant (0: unshifted, ends zeroed -- sub-grid (0,0);
// 1: unshifted 2r+3 taps; 2: shifted): A = filters, S = d/dsigma.
template <int R>
__device__ __forceinline__ void build_tables(const BwParams& p, float4* sA, float4* sS)
{
    constexpr int NT = 2 * R + 3;
    for (int i = threadIdx.x; i < 3 * NT; i += blockDim.x) {
        const int v = i / NT, k = i - v * NT;
        const int f = (v == 2) ? 4 : 0;
        float4 a = make_float4(p.tap[f][k], p.tap[f + 1][k], p.tap[f + 2][k], p.tap[f + 3][k]);
        float4 s = make_float4(p.tap[8 + f][k], p.tap[9 + f][k], p.tap[10 + f][k], p.tap[11 + f][k]);
        if (v == 0 && (k == 0 || k == NT - 1)) {
            a = make_float4(0.f, 0.f, 0.f, 0.f);
            s = a;
        }
        sA[i] = a;
        sS[i] = s;
    }
}

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

// Derivatives at 2x-grid point (rho, kap) as the reference defines them
// (cpu_toed.cpp:204-344): f = sum_{p,q} I(i-p, j-q) X(q) Y(p), with their
// d/dsigma.  FULL: all nine (fx fy fxx fxy fyy fxxy fxyy fxxx fyyy), else fx, fy.
template <int R, bool FULL>
__device__ __forceinline__ void eval_point(const BwImage& im, int rho, int kap, const float4* sA,
                                           const float4* sS, float* d, float* ds)
{
    constexpr int NT = 2 * R + 3;
    int xv, yv;
    variants(rho, kap, &xv, &yv);
    const int i = rho >> 1, j = kap >> 1;
    const float4* XA = sA + xv * NT;
    const float4* XS = sS + xv * NT;
    const float4* YA = sA + yv * NT;
    const float4* YS = sS + yv * NT;
    constexpr int ND = FULL ? 9 : 2;
#pragma unroll
    for (int k = 0; k < ND; ++k) d[k] = ds[k] = 0.f;
    for (int pp = 0; pp < NT; ++pp) {
        const int y = i + R + 1 - pp;  // row i - p, p = pp - (R+1)
        float h0 = 0.f, h1 = 0.f, h2 = 0.f, h3 = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
        for (int qq = 0; qq < NT; ++qq) {
            const float v = pix(im, y, j + R + 1 - qq);
            const float4 t = XA[qq], ts = XS[qq];
            h0 = fmaf(v, t.x, h0);
            h1 = fmaf(v, t.y, h1);
            s0 = fmaf(v, ts.x, s0);
            s1 = fmaf(v, ts.y, s1);
            if (FULL) {
                h2 = fmaf(v, t.z, h2);
                h3 = fmaf(v, t.w, h3);
                s2 = fmaf(v, ts.z, s2);
                s3 = fmaf(v, ts.w, s3);
            }
        }
        const float4 ya = YA[pp], ys = YS[pp];
        // fx = (Gx, G), fy = (G, Gy)
        d[0] = fmaf(h1, ya.x, d[0]);
        ds[0] = fmaf(s1, ya.x, fmaf(h1, ys.x, ds[0]));
        d[1] = fmaf(h0, ya.y, d[1]);
        ds[1] = fmaf(s0, ya.y, fmaf(h0, ys.y, ds[1]));
        if (FULL) {
            d[2] = fmaf(h2, ya.x, d[2]);  // fxx  (Gxx, G)
            ds[2] = fmaf(s2, ya.x, fmaf(h2, ys.x, ds[2]));
            d[3] = fmaf(h1, ya.y, d[3]);  // fxy  (Gx, Gy)
            ds[3] = fmaf(s1, ya.y, fmaf(h1, ys.y, ds[3]));
            d[4] = fmaf(h0, ya.z, d[4]);  // fyy  (G, Gyy)
            ds[4] = fmaf(s0, ya.z, fmaf(h0, ys.z, ds[4]));
            d[5] = fmaf(h2, ya.y, d[5]);  // fxxy (Gxx, Gy)
            ds[5] = fmaf(s2, ya.y, fmaf(h2, ys.y, ds[5]));
            d[6] = fmaf(h1, ya.z, d[6]);  // fxyy (Gx, Gyy)
            ds[6] = fmaf(s1, ya.z, fmaf(h1, ys.z, ds[6]));
            d[7] = fmaf(h3, ya.x, d[7]);  // fxxx (Gxxx, G)
            ds[7] = fmaf(s3, ya.x, fmaf(h3, ys.x, ds[7]));
            d[8] = fmaf(h0, ya.w, d[8]);  // fyyy (G, Gyyy)
            ds[8] = fmaf(s0, ya.w, fmaf(h0, ys.w, ds[8]));
        }
    }
}

template <int R>
__global__ void __launch_bounds__(kBwAdjThreads) bw_adjoint(const __grid_constant__ BwParams p)
{
    constexpr int NT = 2 * R + 3;
    __shared__ float4 sA[3 * NT], sS[3 * NT];
    build_tables<R>(p, sA, sS);
    __syncthreads();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double gsig = 0.0;
    if (e < p.n_edgels) {
        const int k = find_image(p.n_img, e, [&](int i) { return p.img[i].edgel_base; });
        const BwImage& im = p.img[k];
        const int local = e - im.edgel_base;
        const int W2 = 2 * im.W;
        const int gi = im.gidx[local];
        const int rho = gi / W2, kap = gi - (gi / W2) * W2;
        double go[4];
        if (p.out_f64) {
            const double* g = (const double*)im.gout + 4LL * local;
            go[0] = g[0]; go[1] = g[1]; go[2] = g[2]; go[3] = g[3];
        } else {
            const float* g = (const float*)im.gout + 4LL * local;
            go[0] = g[0]; go[1] = g[1]; go[2] = g[2]; go[3] = g[3];
        }
        float d[9], ds[9];
        eval_point<R, true>(im, rho, kap, sA, sS, d, ds);
        // the frozen sector (cpu_toed.cpp:415-462 in closed form)
        const bool xmaj = fabsf(d[0]) >= fabsf(d[1]);
        const int sx = d[0] >= 0.f ? 1 : -1, sy = d[1] >= 0.f ? 1 : -1;
        const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
        const int nr[4] = {rho + ar, rho + sy, rho - ar, rho - sy};  // A+, D+, A-, D-
        const int nc[4] = {kap + ac, kap + sx, kap - ac, kap - sx};
        float nd[4][2], nds[4][2];
#pragma unroll
        for (int q = 0; q < 4; ++q) eval_point<R, false>(im, nr[q], nc[q], sA, sS, nd[q], nds[q]);

        // ---- forward values in FP64 ----
        const double fx = d[0], fy = d[1], fxx = d[2], fxy = d[3], fyy = d[4], fxxy = d[5], fxyy = d[6],
                     fxxx = d[7], fyyy = d[8];
        const double m = sqrt(fx * fx + fy * fy);
        const double nx = fx / m, ny = fy / m;
        const double c = (double)(sx * sy);
        const double t = xmaj ? c * fy / fx : c * fx / fy;  // slope |ny|/|nx| or |nx|/|ny|
        double M[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) M[q] = sqrt((double)nd[q][0] * nd[q][0] + (double)nd[q][1] * nd[q][1]);
        const double fp = M[0] * (1.0 - t) + M[1] * t, fm = M[2] * (1.0 - t) + M[3] * t;
        const double num = fp - fm, den = fm + fp - 2.0 * m;
        const double S = sqrt(1.0 + t * t);
        const double sst = -num * S / (2.0 * den);
        // ---- reverse: position, strength ----
        const double g_sst = 0.5 * (go[0] * nx + go[1] * ny);
        double g_nx = 0.5 * go[0] * sst, g_ny = 0.5 * go[1] * sst;
        const double g_maxf = go[3];  // strength = |max_f| |n| = max_f (max_f > 0 at a maximum)
        const double g_num = g_sst * (-S / (2.0 * den)) + g_maxf * (-num / (4.0 * den));
        const double g_den = g_sst * (num * S / (2.0 * den * den)) + g_maxf * (num * num / (8.0 * den * den));
        double g_t = g_sst * (-num / (2.0 * den)) * t / S;
        double g_m = g_maxf - 2.0 * g_den;
        const double g_fp = g_num + g_den, g_fm = -g_num + g_den;
        const double gM[4] = {g_fp * (1.0 - t), g_fp * t, g_fm * (1.0 - t), g_fm * t};
        g_t += g_fp * (M[1] - M[0]) + g_fm * (M[3] - M[2]);
        double gfx = 0.0, gfy = 0.0;
        if (xmaj) {
            gfx += g_t * (-t / fx);
            gfy += g_t * (c / fx);
        } else {
            gfx += g_t * (c / fy);
            gfy += g_t * (-t / fy);
        }
        const double m3 = m * m * m;
        gfx += g_nx * (1.0 / m - fx * fx / m3) + g_ny * (-fx * fy / m3) + g_m * fx / m;
        gfy += g_nx * (-fx * fy / m3) + g_ny * (1.0 / m - fy * fy / m3) + g_m * fy / m;
        // ---- reverse: orientation atan2(TIx, -TIy) (cpu_toed.cpp:227-232) ----
        const double TIx = fx * (2 * fxx * fxx + 2 * fxy * fxy) + fy * (2 * fxx * fxy + 2 * fyy * fxy) +
                           2 * fx * fy * fxxy + fy * fy * fxyy + fx * fx * fxxx;
        const double TIy = fx * (2 * fxx * fxy + 2 * fyy * fxy) + fy * (2 * fyy * fyy + 2 * fxy * fxy) +
                           2 * fx * fy * fxyy + fx * fx * fxxy + fy * fy * fyyy;
        const double q2 = TIx * TIx + TIy * TIy;
        double gP[9];
        gP[2] = gP[3] = gP[4] = gP[5] = gP[6] = gP[7] = gP[8] = 0.0;
        if (q2 > 0.0 && go[2] != 0.0) {
            const double gX = go[2] * (-TIy) / q2, gY = go[2] * TIx / q2;
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
        gP[0] = gfx;
        gP[1] = gfy;
        float* rec = p.cot + (long long)e * kCotW;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            rec[q] = (float)gP[q];
            gsig += gP[q] * (double)ds[q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double gx = gM[q] * nd[q][0] / M[q], gy = gM[q] * nd[q][1] / M[q];
            rec[9 + 2 * q] = (float)gx;
            rec[10 + 2 * q] = (float)gy;
            gsig += gx * (double)nds[q][0] + gy * (double)nds[q][1];
        }
        rec[17] = __int_as_float((xmaj ? 1 : 0) | (sx > 0 ? 2 : 0) | (sy > 0 ? 4 : 0));
    }
    // dL/dsigma: warp sums, one FP64 atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gsig += __shfl_down_sync(0xffffffffu, gsig, o);
    if ((threadIdx.x & 31) == 0 && gsig != 0.0) atomicAdd(p.gsig, gsig);
}

__device__ __forceinline__ int lower_bound_i(const int* a, int n, int key)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <int R>
__global__ void __launch_bounds__(256) bw_scatter(const __grid_constant__ BwParams p)
{
    constexpr int NT = 2 * R + 3;
    __shared__ float acc[kBwT][kBwT + 1];
    __shared__ float4 sA[3 * NT], sS[3 * NT];
    __shared__ int sList[256];
    __shared__ int sWarp[8], sRange[2];
    __shared__ float sV[8][4][NT];
    build_tables<R>(p, sA, sS);
    const int t = blockIdx.x;
    const int k = find_image(p.n_img, t, [&](int i) { return p.img[i].tile_base; });
    const BwImage& im = p.img[k];
    const int lt = t - im.tile_base;
    const int ty = lt / im.ntx, tx = lt - ty * im.ntx;
    const int i0 = ty * kBwT, j0 = tx * kBwT;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int W2 = 2 * im.W;
    for (int q = tid; q < kBwT * kBwT; q += blockDim.x) acc[q >> 5][q & 31] = 0.f;
    if (tid == 0) {
        // edgels whose windows can reach the tile: original row of P in [i0-R-2, i0+kBwT+R+2)
        const int r0 = max(0, 2 * (i0 - R - 2)), r1 = min(2 * im.H, 2 * (i0 + kBwT + R + 2));
        sRange[0] = lower_bound_i(im.gidx, im.n, r0 * W2);
        sRange[1] = lower_bound_i(im.gidx, im.n, r1 * W2);
    }
    __syncthreads();
    const int lo = sRange[0], hi = sRange[1];
    const int clo = j0 - R - 2, chi = j0 + kBwT + R + 2;
    for (int base = lo; base < hi; base += 256) {
        const int e = base + tid;
        bool rel = false;
        if (e < hi) {
            const int kap = im.gidx[e] % W2;
            const int j = kap >> 1;
            rel = (j >= clo && j < chi);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, rel);
        if (lane == 0) sWarp[wid] = __popc(bal);
        __syncthreads();
        int off = 0, cnt = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) {
            off += (w < wid) ? sWarp[w] : 0;
            cnt += sWarp[w];
        }
        if (rel) sList[off + __popc(bal & ((1u << lane) - 1u))] = e;
        __syncthreads();
        // jobs: (edgel, point) pairs, one warp each
        for (int job = wid; job < cnt * 5; job += 8) {
            const int el = sList[job / 5], pt = job - (job / 5) * 5;
            const int gi = im.gidx[el];
            int rho = gi / W2, kap = gi - (gi / W2) * W2;
            const float* rec = p.cot + (long long)(im.edgel_base + el) * kCotW;
            const int bits = __float_as_int(rec[17]);
            const bool xmaj = bits & 1;
            const int sx = (bits & 2) ? 1 : -1, sy = (bits & 4) ? 1 : -1;
            const int ar = xmaj ? 0 : sy, ac = xmaj ? sx : 0;
            if (pt == 1) { rho += ar; kap += ac; }
            else if (pt == 2) { rho += sy; kap += sx; }
            else if (pt == 3) { rho -= ar; kap -= ac; }
            else if (pt == 4) { rho -= sy; kap -= sx; }
            int xv, yv;
            variants(rho, kap, &xv, &yv);
            // y-vectors per x filter: V_f(p) = sum_k g_k Y_k(p)
            if (lane < NT) {
                const float4 y = sA[yv * NT + lane];
                float v0, v1, v2 = 0.f, v3 = 0.f;
                if (pt == 0) {
                    v0 = rec[1] * y.y + rec[4] * y.z + rec[8] * y.w;  // G  x (fy, fyy, fyyy)
                    v1 = rec[0] * y.x + rec[3] * y.y + rec[6] * y.z;  // Gx x (fx, fxy, fxyy)
                    v2 = rec[2] * y.x + rec[5] * y.y;                 // Gxx x (fxx, fxxy)
                    v3 = rec[7] * y.x;                                // Gxxx x fxxx
                } else {
                    v0 = rec[8 + 2 * pt] * y.y;  // fy at the neighbour
                    v1 = rec[7 + 2 * pt] * y.x;  // fx at the neighbour
                }
                sV[wid][0][lane] = v0;
                sV[wid][1][lane] = v1;
                sV[wid][2][lane] = v2;
                sV[wid][3][lane] = v3;
            }
            __syncwarp();
            // window rows i - p, cols j - q (p = pp - R - 1) intersected with the tile
            const int i = rho >> 1, j = kap >> 1;
            const int pp0 = max(0, i + R + 1 - (i0 + kBwT - 1)), pp1 = min(NT - 1, i + R + 1 - i0);
            const int qq0 = max(0, j + R + 1 - (j0 + kBwT - 1)), qq1 = min(NT - 1, j + R + 1 - j0);
            const int nrr = pp1 - pp0 + 1, ncc = qq1 - qq0 + 1;
            if (nrr > 0 && ncc > 0) {
                for (int z = lane; z < nrr * ncc; z += 32) {
                    const int pp = pp0 + z / ncc, qq = qq0 + z - (z / ncc) * ncc;
                    const float4 x = sA[xv * NT + qq];
                    const float v = x.x * sV[wid][0][pp] + x.y * sV[wid][1][pp] + x.z * sV[wid][2][pp] +
                                    x.w * sV[wid][3][pp];
                    atomicAdd(&acc[i + R + 1 - pp - i0][j + R + 1 - qq - j0], v);
                }
            }
            __syncwarp();
        }
        __syncthreads();
    }
    for (int q = tid; q < kBwT * kBwT; q += blockDim.x) {
        const int y = i0 + (q >> 5), x = j0 + (q & 31);
        if (y < im.H && x < im.W) im.gpix[(long long)y * im.W + x] = acc[q >> 5][q & 31];
    }
}

template <int R>
static cudaError_t launch_bw(const BwParams& p, cudaStream_t stream)
{
    void* args[] = {const_cast<BwParams*>(&p)};
    cudaError_t e = cudaSuccess;
    if (p.n_edgels > 0)
        e = cudaLaunchKernel((const void*)bw_adjoint<R>, dim3((p.n_edgels + kBwAdjThreads - 1) / kBwAdjThreads),
                             dim3(kBwAdjThreads), args, 0, stream);
    if (e == cudaSuccess) e = cudaLaunchKernel((const void*)bw_scatter<R>, dim3(p.n_tiles), dim3(256), args, 0, stream);
    return e;
}

cudaError_t backward_launch(const toed_grad_image* items, int n, const toed_params* prm, int r, float* cot,
                            double* gsig, cudaStream_t stream)
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
    p.cot = cot;
    p.gsig = gsig;
    int edg = 0, tiles = 0;
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
        d.ntx = (d.W + kBwT - 1) / kBwT;
        d.nty = (d.H + kBwT - 1) / kBwT;
        d.tile_base = tiles;
        edg += d.n;
        tiles += d.ntx * d.nty;
    }
    p.n_edgels = edg;
    p.n_tiles = tiles;
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
