// toed_common.cuh -- launch descriptors shared by the detection kernels and
// the host side of the C ABI.
//
// Data layout in HBM (all caller-owned except the scratch block):
//   image k      : H x pitch pixels (uint8 or float32), row-major
//   edgels k     : capacity x 4 (float32 or float64) [x, y, orientation, strength]
//   scratch      : work-queue / cursor / flags words, staging records
//                  (double4 + int index per edgel), the row-segment table
//                  (int2 {staging offset, count} per (2x-grid row, strip column)),
//                  and the ordering pass' tile sums.
#pragma once
#include <cstdint>
#include <cuda.h>  // CUtensorMap (the type only; encoding goes through the runtime's driver entry point)
#include <cuda_runtime.h>

#include "../../include/toed_gb300.h"

namespace toed {

constexpr int kMaxTaps = 2 * TOED_MAX_RADIUS + 3;  // taps of the widest (shifted/full) filter
constexpr int kBatchMax = 64;                      // images per launch (larger batches are chunked)
constexpr int kSizeClasses = 48;                   // launch size classes floor(log2(pixels)) of tuned shapes
constexpr int kThreads = 256;                      // threads per detection CTA
constexpr int kExt = 32;                           // strip width incl. a 1-pixel ring each side
constexpr int kInner = kExt - 2;                   // 30 output columns per strip
constexpr int kHalves = kExt / 32;                 // warp-wide column groups of a strip
constexpr int kRawRowBytes = 256;                  // bytes per staged input row (TMA box row) at most
constexpr int kStepRows = 16;                      // original rows per sliding step (B)
constexpr int kColRows = 8;                        // rows per column-pass thread (register blocking)
constexpr int kSegTile = 1024;                     // segments per ordering-pass tile
constexpr int kStageBlk = 256;                     // staging records a CTA reserves at a time
// Edgels whose third-order vector cancels by more than this factor (sum of
// the terms' magnitudes over the largest component) get their orientation
// recomputed from the image in FP64 (HYBRID precision, grid orientation).
constexpr float kRefineKappa = 20.f;
// Default bound of the wait for a copy group's ready flag (polls ~256 ns
// apart: a few seconds), after which the kernel flags TOED_FLAG_TIMEOUT and
// skips the units whose pixels have not arrived (BatchParams::ready_spins).
constexpr int kReadySpinLimit = 1 << 24;

// Bounds-checked builds (-DTOED_DEBUG_BOUNDS, a separate debug library):
// TOED_IN_BOUNDS(cond, words) guards a shared- or global-memory access; a
// failed check skips the access, sets TOED_FLAG_BOUNDS in words[2] and
// records the source line of the first failure in words[4] -- a status the
// host reads, never a trap.  In release builds the macro is `true` and every
// guard compiles away.
#ifdef TOED_DEBUG_BOUNDS
__device__ __forceinline__ bool debug_in_bounds(bool ok, int* words, int line)
{
    if (!ok) {
        atomicOr(&words[2], TOED_FLAG_BOUNDS);
        atomicCAS(&words[4], 0, line);
    }
    return ok;
}
#define TOED_IN_BOUNDS(cond, words) ::toed::debug_in_bounds((cond), (words), __LINE__)
#else
#define TOED_IN_BOUNDS(cond, words) true
#endif
constexpr int kWords = 8;  // scratch words: [0] queue [1] cursor [2] flags [3] refine length [4] first bad line

// 1-D taps, index k <-> offset x = k - (r+1) (+0.5 for the shifted set).
// Filters: 0 G, 1 Gx, 2 Gxx, 3 Gxxx, 4..7 the same shifted by +0.5.
// Passed by value as a kernel parameter, so unrolled loops read each tap as
// a constant-bank operand of the FMA.
struct TapBlock {
    float v[8][kMaxTaps];
};

// The same taps in FP64, for the orientation recomputation.
struct TapBlock64 {
    double v[8][kMaxTaps];
};

struct DetImage {
    const void* src;
    long long pitch;     // elements
    void* out;           // edgels
    int* count;          // user count word
    int* index;          // optional grid index output
    long long seg_base;  // first segment of this image (tile aligned)
    long long nseg;      // segments of this image (rows x strip/tile columns)
    int H, W;
    int dtype;
    int cap;
    int nsc, nsr;        // strip columns / strip rows
    int S;               // strip inner rows of this image's work units (multiple of kStepRows minus 2)
    int unit_base;       // first work unit
    int tile_base;       // first ordering tile
    int tma;             // 1: rows arrive by TMA through BatchParams::tmap[k]; 2: by per-thread async
                         // copies (float32, any address); 0: plain loads
    int tma_align;       // element alignment of a TMA box's x coordinate (16 bytes)
    int tma_boxw;        // box width in elements (the halo row plus the alignment shift)
    int wait_slot;       // 0: pixels ready at launch; g > 0: the copy engine is still bringing them in,
                         // BatchParams::ready[g - 1] reads ready_epoch once they are complete
};

struct Scratch {
    int* words;          // kWords: [0] unit queue, [1] staging cursor, [2] flags, [3] refine-list length,
                         // [4] (bounds-checked builds) source line of the first failed check
    double4_32a* staging;  // staged edgels: TO correction (x, y, orientation, strength); the
                           // detection uses the same memory as float4 records (det_stage)
    int* staging_idx;
    long long staging_cap;
    int2* seg;           // per segment {staging offset, count}
    long long seg_cap;   // segments `seg` holds
    int* tile_sum;       // per ordering tile
    long long* img_base; // per image: exclusive prefix of its first segment
    int4* refine;        // edgels whose orientation is recomputed in FP64: {staging slot, image, Gr, Gc}
    int refine_cap;      // entries of `refine` (0: no recomputation)
};

// The detection's staged edgel: a float4 in the staging memory beside the
// 2x-grid index in staging_idx (20 bytes per edgel).  x, y hold what the
// output's FP64 position is rebuilt from without loss: in HYBRID precision
// the subpixel offset 0.5 s* n (the grid part 0.5 (G - 1) is exact), in
// FP32 precision the FP32 position G + s* n on the 2x grid; then the
// orientation and the strength.
__device__ __forceinline__ float4* det_stage(const Scratch& sc) { return reinterpret_cast<float4*>(sc.staging); }

// Output position (x, y) = ((pos - 1) / 2) of a staged edgel (cpu_toed.cpp:516-521).
__device__ __forceinline__ double2 det_xy(const float4& rec, int idx, int W2, bool hyb)
{
    const int Gr = idx / W2, Gc = idx - Gr * W2;
    if (hyb)
        return make_double2((double)(0.5f * (float)(Gc - 1)) + (double)rec.x,
                            (double)(0.5f * (float)(Gr - 1)) + (double)rec.y);
    return make_double2(((double)rec.x - 1.0) * 0.5, ((double)rec.y - 1.0) * 0.5);
}

struct BatchParams {
    CUtensorMap tmap[kBatchMax];  // per image: 2-D map, box (tma_boxw x kStepRows), OOB zero fill
    TapBlock taps;
    TapBlock64 taps64;
    float thr;
    float thr2;          // candidate prefilter on |grad I|^2: a little below thr^2 (-1 when thr < 0)
    int border;
    int S;               // strip inner rows of most work units (multiple of kStepRows minus 2); the
                         // images at the end of the queue may use shorter ones (DetImage::S)
    int n_img;
    int n_units;
    int n_tiles;
    int out_f64;
    int radius;
    int stage_blk;       // staging records reserved per atomic (1: exactly each step's edgels)
    int hyb;             // 1: peak fit on exact FP32 differences, FP64 recomputation of ill-conditioned
                         // orientations (TOED_HYBRID)
    int qad;             // 1: orientation from derivatives interpolated at the subpixel point (TOED_ORI_QAD)
    int nms_to;          // 1: NMS and peak fit along the corrected normal (TOED_NMS_TO_NORMAL)
    int det_rec;         // ordering pass input: 1 the detection's float4 records (det_stage), 0 the TO
                         // correction's double4 records
    const int* ready;    // per copy group: ready_epoch once the group's images are in device memory
    int ready_epoch;
    int ready_spins;     // polls of a ready flag before the wait gives up (TOED_FLAG_TIMEOUT)
    Scratch sc;
    DetImage img[kBatchMax];
};
static_assert(sizeof(BatchParams) <= 32764, "BatchParams is passed as one kernel parameter");

// Block-wide exclusive scan of one int per thread (NT threads); leaves the
// block total in *total.  s_warp: 33 ints of shared memory.
template <int NT>
__device__ __forceinline__ int block_excl_scan(int v, int* s_warp, int* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        constexpr int NW = NT / 32;
        int w = (lane < NW) ? s_warp[lane] : 0;
        int wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        if (lane < NW) s_warp[lane] = wi - w;
        if (lane == NW - 1) s_warp[32] = wi;
    }
    __syncthreads();
    const int r = incl - v + s_warp[wid];
    *total = s_warp[32];
    __syncthreads();
    return r;
}

// Index of the image whose [base, next base) range holds `u` (bases ascending).
template <typename GetBase>
__device__ __forceinline__ int find_image(int n_img, int u, GetBase base)
{
    int lo = 0, hi = n_img - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (base(mid) <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace toed
