// toed_finalize.cu -- ordering pass: turns the detection kernel's staged
// edgels and row-segment table into each image's edgel list in the
// reference's order (row-major over the 2x grid, cpu_toed.cpp:510-538).
//
// Segments are (2x-grid row, strip column) pairs laid out row-major per image
// and padded to whole tiles of kSegTile.  Three short kernels:
//   fin_tile_sums : edgels per tile; then the FP64 orientation recomputation
//                   of the edgels the detection kernel listed
//   fin_tile_scan : exclusive scan over tiles; per-image base and count,
//                   capacity flag
//   fin_scatter   : per tile, scan the segment counts, then copy the tile's
//                   staged records cooperatively to their list positions
//                   (global prefix - image base), converting to the output
//                   dtype.
#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

// One listed edgel, one warp: the nine derivatives at 2x-grid point
// (Gr, Gc) = (2i + a, 2j + b) straight from the image with FP64 taps, zero
// outside the image -- the (2r+1)^2 window of unshifted taps on sub-grid
// (0, 0) (cpu_toed.cpp:205-221), the (2r+3)^2 window with the half-pixel
// shifted taps along the odd axes elsewhere (cpu_toed.cpp:246-344) -- then the
// third-order vector (cpu_toed.cpp:227-232) and its angle in FP64, written
// over the staged orientation.  Lane t forms the four column-filtered sums of
// window row t; the row filters then weight them and the warp reduces.
constexpr int kRefineChunk = 9;

__device__ void refine_edgel(const BatchParams& p, int4 e, int lane)
{
    const DetImage& im = p.img[e.y];
    const int r = p.radius;
    const int i = e.z >> 1, a = e.z & 1, j = e.w >> 1, b = e.w & 1;
    const int h = (a | b) ? r + 1 : r;
    const double* X = &p.taps64.v[b ? 4 : 0][0];  // filter f, tap k: X[f * kMaxTaps + k]
    const double* Y = &p.taps64.v[a ? 4 : 0][0];
    const int dp = lane - h, row = i - dp;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0, y0 = 0.0, y1 = 0.0, y2 = 0.0, y3 = 0.0;
    if (lane <= 2 * h && row >= 0 && row < im.H) {
        // the row in chunks of kRefineChunk columns, each chunk's loads
        // first (independent, so in flight together)
        const long long ro = (long long)row * im.pitch;
        const bool u8 = im.dtype == TOED_U8;
        const int k0 = r + 1 - h;  // tap of column offset q = -h
        for (int c0 = 0; c0 <= 2 * h; c0 += kRefineChunk) {
            float v[kRefineChunk];
#pragma unroll
            for (int t = 0; t < kRefineChunk; ++t) {
                const int col = j + h - (c0 + t);  // column offset q = c0 + t - h
                v[t] = 0.f;
                if (c0 + t <= 2 * h && col >= 0 && col < im.W)
                    v[t] = u8 ? (float)static_cast<const unsigned char*>(im.src)[ro + col]
                              : static_cast<const float*>(im.src)[ro + col];
            }
#pragma unroll
            for (int t = 0; t < kRefineChunk; ++t) {
                if (c0 + t > 2 * h) break;
                const double x = v[t];
                const int kq = k0 + c0 + t;
                s0 = fma(x, X[kq], s0);
                s1 = fma(x, X[kMaxTaps + kq], s1);
                s2 = fma(x, X[2 * kMaxTaps + kq], s2);
                s3 = fma(x, X[3 * kMaxTaps + kq], s3);
            }
        }
        const int kp = dp + r + 1;
        y0 = Y[kp];
        y1 = Y[kMaxTaps + kp];
        y2 = Y[2 * kMaxTaps + kp];
        y3 = Y[3 * kMaxTaps + kp];
    }
    // fx fy fxx fxy fyy fxxy fxyy fxxx fyyy
    double d[9] = {y0 * s1, y1 * s0, y0 * s2, y1 * s1, y2 * s0, y1 * s2, y2 * s1, y0 * s3, y3 * s0};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int f = 0; f < 9; ++f) d[f] += __shfl_xor_sync(0xffffffffu, d[f], o);
    if (lane == 0) {
        const double fx = d[0], fy = d[1], fxx = d[2], fxy = d[3], fyy = d[4], fxxy = d[5], fxyy = d[6],
                     fxxx = d[7], fyyy = d[8];
        const double tix = fx * (2 * fxx * fxx + 2 * fxy * fxy) + fy * (2 * fxx * fxy + 2 * fyy * fxy) +
                           2 * fx * fy * fxxy + fy * fy * fxyy + fx * fx * fxxx;
        const double tiy = fx * (2 * fxx * fxy + 2 * fyy * fxy) + fy * (2 * fyy * fyy + 2 * fxy * fxy) +
                           2 * fx * fy * fxyy + fx * fx * fxxy + fy * fy * fyyy;
        const double ori = (tix == 0.0 && tiy == 0.0) ? __longlong_as_double(0x7ff8000000000000LL) : atan2(tix, -tiy);
        det_stage(p.sc)[e.x].z = (float)ori;
    }
}

__global__ void __launch_bounds__(256) fin_tile_sums(const __grid_constant__ BatchParams p)
{
    __shared__ int s_warp[33];
    const int t = blockIdx.x;
    const int k = find_image(p.n_img, t, [&](int i) { return p.img[i].tile_base; });
    const DetImage& im = p.img[k];
    const long long nseg = im.nseg;
    const long long first = (long long)(t - im.tile_base) * kSegTile;
    int sum = 0;
    for (int i = threadIdx.x; i < kSegTile; i += blockDim.x) {
        const long long q = first + i;
        if (q < nseg) sum += p.sc.seg[im.seg_base + q].y;
    }
    int total;
    block_excl_scan<256>(sum, s_warp, &total);
    if (threadIdx.x == 0) p.sc.tile_sum[t] = total;
    if (p.sc.refine_cap > 0) {
        const int nref = min(p.sc.words[3], p.sc.refine_cap);
        // entry q to warp q / gridDim of block q % gridDim: a short list
        // spreads over all SMs' FP64 pipes
        const int lane = threadIdx.x & 31, w = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
        for (int q = w; q < nref; q += gridDim.x * 8) refine_edgel(p, p.sc.refine[q], lane);
    }
}

__global__ void __launch_bounds__(1024) fin_tile_scan(const __grid_constant__ BatchParams p)
{
    __shared__ int s_warp[33];
    int carry = 0;
    for (int base = 0; base < p.n_tiles; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = (i < p.n_tiles) ? p.sc.tile_sum[i] : 0;
        int total;
        const int ex = block_excl_scan<1024>(v, s_warp, &total);
        if (i < p.n_tiles) p.sc.tile_sum[i] = carry + ex;
        carry += total;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < p.n_img; k += blockDim.x) {
        const long long b0 = p.sc.tile_sum[p.img[k].tile_base];
        const long long b1 = (k + 1 < p.n_img) ? p.sc.tile_sum[p.img[k + 1].tile_base] : carry;
        const int cnt = (int)(b1 - b0);
        p.sc.img_base[k] = b0;
        *p.img[k].count = cnt;
        if (cnt > p.img[k].cap) atomicOr(&p.sc.words[2], TOED_FLAG_OVER_CAPACITY);
    }
    if (threadIdx.x == 0) p.sc.words[3] = 0;  // refine list empty for the next launch (fin_tile_sums has read it)
}

// One CTA per tile of kSegTile segments: an exclusive scan gives every
// segment its place in the image's list; then the tile's records are copied
// cooperatively -- thread t copies records t, t+256, ... of the tile, finding
// the owning segment by binary search over the scanned offsets -- so writes
// are coalesced and no thread serialises a long segment.
constexpr int kFinThreads = 256;
constexpr int kSegPerThread = kSegTile / kFinThreads;

__global__ void __launch_bounds__(kFinThreads) fin_scatter(const __grid_constant__ BatchParams p)
{
    __shared__ int s_warp[33];
    __shared__ int s_dst[kSegTile];      // exclusive prefix of counts within the tile
    __shared__ int s_src[kSegTile];      // staging offset of each segment
    const int t = blockIdx.x;
    const int k = find_image(p.n_img, t, [&](int i) { return p.img[i].tile_base; });
    const DetImage& im = p.img[k];
    const long long q0 = (long long)(t - im.tile_base) * kSegTile + threadIdx.x * kSegPerThread;
    int cnt[kSegPerThread], sum = 0;
#pragma unroll
    for (int u = 0; u < kSegPerThread; ++u) {
        const long long q = q0 + u;
        const int2 sg = (q < im.nseg) ? p.sc.seg[im.seg_base + q] : make_int2(0, 0);
        cnt[u] = sg.y;
        s_src[threadIdx.x * kSegPerThread + u] = sg.x;
        sum += sg.y;
    }
    int total;
    int run = block_excl_scan<kFinThreads>(sum, s_warp, &total);
#pragma unroll
    for (int u = 0; u < kSegPerThread; ++u) {
        s_dst[threadIdx.x * kSegPerThread + u] = run;
        run += cnt[u];
    }
    __syncthreads();
    const long long base = (long long)p.sc.tile_sum[t] - p.sc.img_base[k];  // list position of the tile
    const long long cap = im.cap;
    for (int r = threadIdx.x; r < total; r += kFinThreads) {
        int lo = 0, hi = kSegTile - 1;  // last segment with s_dst <= r
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_dst[mid] <= r) lo = mid; else hi = mid - 1;
        }
        const long long d = base + r, src = (long long)s_src[lo] + (r - s_dst[lo]);
        if (d >= cap || src >= p.sc.staging_cap) continue;
        double4_32a rc;
        int gi = 0;
        if (p.det_rec) {  // the detection's compact record
            const float4 st = det_stage(p.sc)[src];
            gi = p.sc.staging_idx[src];
            const double2 xy = det_xy(st, gi, 2 * im.W, p.hyb != 0);
            rc = make_double4_32a(xy.x, xy.y, (double)st.z, (double)st.w);
        } else {
            rc = p.sc.staging[src];
            if (im.index) gi = p.sc.staging_idx[src];
        }
        if (p.out_f64) {  // two 16-byte stores: the caller's buffer need only be 16-byte aligned
            double2* o = reinterpret_cast<double2*>(im.out) + 2 * d;
            o[0] = make_double2(rc.x, rc.y);
            o[1] = make_double2(rc.z, rc.w);
        } else {
            reinterpret_cast<float4*>(im.out)[d] = make_float4((float)rc.x, (float)rc.y, (float)rc.z, (float)rc.w);
        }
        if (im.index) im.index[d] = gi;
    }
}

cudaError_t preload_finalize(int radius, bool qad)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, (const void*)fin_tile_sums);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)fin_tile_scan);
    if (e == cudaSuccess) e = qad ? preload_scatter_qad(radius) : cudaFuncGetAttributes(&fa, (const void*)fin_scatter);
    return e;
}

cudaError_t launch_finalize(const BatchParams& p, cudaStream_t stream)
{
    void* args[] = {const_cast<BatchParams*>(&p)};
    cudaError_t e = cudaLaunchKernel((const void*)fin_tile_sums, dim3(p.n_tiles), dim3(256), args, 0, stream);
    if (e != cudaSuccess) return e;
    e = cudaLaunchKernel((const void*)fin_tile_scan, dim3(1), dim3(1024), args, 0, stream);
    if (e != cudaSuccess) return e;
    if (p.qad) return launch_scatter_qad(p, stream);
    return cudaLaunchKernel((const void*)fin_scatter, dim3(p.n_tiles), dim3(kFinThreads), args, 0, stream);
}

}  // namespace toed
