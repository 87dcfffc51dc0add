// toed_finalize.cu -- ordering pass: turns the detection kernel's staged
// edgels and row-segment table into each image's edgel list in the
// reference's order (row-major over the 2x grid, cpu_toed.cpp:510-538).
//
// Segments are (2x-grid row, strip column) pairs laid out row-major per image
// and padded to whole tiles of kSegTile.  Three short kernels:
//   fin_tile_sums : edgels per tile
//   fin_tile_scan : exclusive scan over tiles; per-image base and count,
//                   capacity flag
//   fin_scatter   : per tile, scan the segment counts, then copy the tile's
//                   staged records cooperatively to their list positions
//                   (global prefix - image base), converting to the output
//                   dtype.
#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {

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
        const double4_32a rc = p.sc.staging[src];
        if (p.out_f64) {  // two 16-byte stores: the caller's buffer need only be 16-byte aligned
            double2* o = reinterpret_cast<double2*>(im.out) + 2 * d;
            o[0] = make_double2(rc.x, rc.y);
            o[1] = make_double2(rc.z, rc.w);
        } else {
            reinterpret_cast<float4*>(im.out)[d] = make_float4((float)rc.x, (float)rc.y, (float)rc.z, (float)rc.w);
        }
        if (im.index) im.index[d] = p.sc.staging_idx[src];
    }
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
