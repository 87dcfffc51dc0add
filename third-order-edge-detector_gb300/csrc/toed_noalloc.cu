// toed_noalloc.cu -- toed_detect_noalloc: single-image detection that makes
// no device (or host heap) allocation of its own.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// detect edges -- code running under a memory pool or allocator that owns
// all device memory (an inference server's arena, a real-time loop that
// forbids allocation after start-up, a plug-in host that hands out only
// pre-sized buffers) -- and so cannot create a toed_ctx, whose scratch grows
// with cudaMalloc on demand.
//
// How: the scratch the fused kernel and the ordering pass need (work-queue
// and flag words, staged edgel records, the row-segment table, tile sums)
// lives in one file-scope __device__ array of fixed size, g_noalloc_scratch.
// The CUDA runtime loads the module that holds it lazily (the default since
// CUDA 12): the bytes are reserved on a device when the first call on that
// device looks the array up, and stay reserved until the process exits.
// Host code may not use the array's name as a device address (on the host it
// names a host-side stand-in), so that first call looks the device address
// up with cudaGetSymbolAddress, with the device current, and caches it with
// the device's SM count and the kernels' occupancy.  Make the first call on
// each device at start-up -- before a pool or arena claims the device's
// memory (else it returns TOED_ERR_CUDA) and before any stream capture that
// includes this entry point.
//
// Limits: an image of at most TOED_NOALLOC_MAX_DIM rows and columns and
// TOED_NOALLOC_MAX_PIXELS pixels, and an edgel capacity of at most
// TOED_NOALLOC_MAX_EDGELS; larger requests return TOED_ERR_CAPACITY before
// anything is launched.  All calls share the one array and it keeps the
// previous call's contents: each call clears the queue / cursor / flag words
// it needs at zero (an asynchronous memset on the caller's stream), and calls
// whose work overlaps on the GPU (different streams, or different host
// threads on the same device) race on the array and corrupt each other's
// results -- serialise them.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {
void make_taps(double sigma, int r, TapBlock* tb);
void make_taps64(double sigma, int r, TapBlock64* tb);

namespace {

constexpr long long kNaMaxPixels = TOED_NOALLOC_MAX_PIXELS;
constexpr int kNaMaxDim = TOED_NOALLOC_MAX_DIM;
constexpr long long kNaMaxEdgels = TOED_NOALLOC_MAX_EDGELS;
// segments 2H x ceil(W/30) <= pixels/15 + 2H, padded to whole ordering tiles
constexpr long long kNaMaxTiles = (kNaMaxPixels / 15 + 2LL * kNaMaxDim) / kSegTile + 2;
constexpr long long kNaMaxSegs = kNaMaxTiles * kSegTile;
constexpr long long kNaRefine = kNaMaxEdgels / 64 + 1024;  // orientation recomputation list

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffWords = 0;
constexpr size_t kOffStaging = align256(kOffWords + kWords * sizeof(int));
constexpr size_t kOffIdx = align256(kOffStaging + sizeof(double4_32a) * kNaMaxEdgels);
constexpr size_t kOffSeg = align256(kOffIdx + sizeof(int) * kNaMaxEdgels);
constexpr size_t kOffTiles = align256(kOffSeg + sizeof(int2) * kNaMaxSegs);
constexpr size_t kOffBase = align256(kOffTiles + sizeof(int) * kNaMaxTiles);
constexpr size_t kOffRefine = align256(kOffBase + sizeof(long long));
constexpr size_t kScratchBytes = align256(kOffRefine + sizeof(int4) * kNaRefine);

// The fixed scratch (see the file comment): about 11 MB per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_dev_scratch[kMaxDevices] = {};
int g_dev_sms[kMaxDevices] = {};
int g_dev_bps[kMaxDevices][TOED_MAX_RADIUS + 1][2][2] = {};  // resident CTAs per SM [radius][hybrid][TO normal]

// Device address of g_noalloc_scratch on `dev` (current), the device's SM
// count and the detection kernel's occupancy, looked up once per device
// (and radius / precision) so that later calls make no such queries.
cudaError_t device_setup(int dev, int r, bool hyb, bool nmsto, const DetectEntry& ent, unsigned char** base, int* sms,
                         int* bps)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_dev_scratch[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        g_dev_sms[dev] = n;
        g_dev_scratch[dev] = static_cast<unsigned char*>(ptr);
    }
    int& b = g_dev_bps[dev][r][hyb ? 1 : 0][nmsto ? 1 : 0];
    if (b == 0) {
        cudaError_t e = cudaFuncSetAttribute(ent.func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ent.smem);
        if (e != cudaSuccess) return e;
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ent.func, kThreads, ent.smem);
        if (e != cudaSuccess) return e;
        if (n <= 0) return cudaErrorInvalidConfiguration;
        b = n;
    }
    *base = g_dev_scratch[dev];
    *sms = g_dev_sms[dev];
    *bps = b;
    return cudaSuccess;
}

}  // namespace
}  // namespace toed

using namespace toed;

extern "C" toed_status toed_detect_noalloc(const toed_image* im, const toed_params* prm, cudaStream_t stream)
{
    if (!im || !prm) return TOED_ERR_INVALID_ARG;
    // the same image checks as toed_detect (pointers, sizes, dtype, alignment)
    const toed_status ist = check_image(*im);
    if (ist != TOED_OK) return ist;
    if (!(prm->sigma > 0.f) || !std::isfinite(prm->sigma) || !std::isfinite(prm->threshold) || prm->border < 1)
        return TOED_ERR_INVALID_ARG;
    if (prm->out_dtype != TOED_F32 && prm->out_dtype != TOED_F64) return TOED_ERR_INVALID_ARG;
    if (prm->precision != TOED_HYBRID && prm->precision != TOED_FP32) return TOED_ERR_INVALID_ARG;
    if (prm->orientation != TOED_ORI_GRID && prm->orientation != TOED_ORI_QAD) return TOED_ERR_INVALID_ARG;
    if (prm->nms_direction != TOED_NMS_GRADIENT && prm->nms_direction != TOED_NMS_TO_NORMAL)
        return TOED_ERR_INVALID_ARG;
    if (prm->nms_direction == TOED_NMS_TO_NORMAL && prm->orientation != TOED_ORI_GRID) return TOED_ERR_UNSUPPORTED;
    // the fixed scratch bounds the image and the edgel capacity
    if (im->height > kNaMaxDim || im->width > kNaMaxDim || (long long)im->height * im->width > kNaMaxPixels ||
        im->capacity > kNaMaxEdgels)
        return TOED_ERR_CAPACITY;
    const int r = prm->radius > 0 ? prm->radius : (int)std::ceil(4.0 * (double)prm->sigma);
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    const bool nmsto = prm->nms_direction == TOED_NMS_TO_NORMAL;
    const DetectEntry ent = detect_entry(r, prm->precision != TOED_FP32, false, nmsto);
    if (!ent.func) return TOED_ERR_UNSUPPORTED;

    int dev = 0, sms = 0, bps = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TOED_ERR_CUDA;
    unsigned char* base = nullptr;
    if (device_setup(dev, r, prm->precision != TOED_FP32, nmsto, ent, &base, &sms, &bps) != cudaSuccess)
        return TOED_ERR_CUDA;

    BatchParams p;  // on the stack: no heap allocation either
    std::memset(&p, 0, sizeof(p));
    make_taps((double)prm->sigma, r, &p.taps);
    make_taps64((double)prm->sigma, r, &p.taps64);
    p.thr = prm->threshold;
    p.thr2 = prm->threshold < 0.f ? -1.f : prm->threshold * prm->threshold * 0.9999f;
    p.border = prm->border;
    p.n_img = 1;
    p.out_f64 = prm->out_dtype == TOED_F64;
    p.radius = r;
    p.hyb = prm->precision != TOED_FP32 ? 1 : 0;
    p.qad = prm->orientation == TOED_ORI_QAD ? 1 : 0;
    p.nms_to = nmsto ? 1 : 0;
    p.det_rec = 1;
    p.stage_blk = 1;  // staging sized to the capacity exactly: reserve each step's edgels alone
    // strip height: the tallest of 254 / 126 / 62 / 30 / 14 rows that still
    // gives every resident CTA a few strips
    const int nsc = (im->width + kInner - 1) / kInner;
    const long long resident = (long long)bps * sms;
    int S = kStepRows - 2;
    for (int st = 16; st >= 1; st /= 2) {
        const int s = st * kStepRows - 2;
        if ((long long)nsc * ((im->height + s - 1) / s) >= 4 * resident) {
            S = s;
            break;
        }
    }
    p.S = S;
    DetImage& d = p.img[0];
    d.src = im->pixels;
    d.pitch = im->pitch;
    d.out = im->edgels;
    d.count = im->count;
    d.index = im->grid_index;
    d.H = im->height;
    d.W = im->width;
    d.dtype = im->dtype;
    d.cap = im->capacity;
    d.nsc = nsc;
    d.S = S;
    d.nsr = (im->height + S - 1) / S;
    d.unit_base = 0;
    d.tile_base = 0;
    d.seg_base = 0;
    d.nseg = 2LL * im->height * nsc;
    encode_rows_map(&p.tmap[0], d, r);
    p.n_units = d.nsc * d.nsr;
    p.n_tiles = (int)((d.nseg + kSegTile - 1) / kSegTile);
    p.sc.words = reinterpret_cast<int*>(base + kOffWords);
    p.sc.staging = reinterpret_cast<double4_32a*>(base + kOffStaging);
    p.sc.staging_idx = reinterpret_cast<int*>(base + kOffIdx);
    p.sc.staging_cap = im->capacity > 0 ? im->capacity : 1;
    p.sc.seg = reinterpret_cast<int2*>(base + kOffSeg);
    p.sc.seg_cap = kNaMaxSegs;
    p.sc.tile_sum = reinterpret_cast<int*>(base + kOffTiles);
    p.sc.img_base = reinterpret_cast<long long*>(base + kOffBase);
    p.sc.refine = reinterpret_cast<int4*>(base + kOffRefine);
    p.sc.refine_cap = (p.hyb && !p.qad) ? (int)kNaRefine : 0;

    // queue, staging cursor, flags and refine-list length start at zero on every call
    if (cudaMemsetAsync(p.sc.words, 0, kWords * sizeof(int), stream) != cudaSuccess) return TOED_ERR_CUDA;
    const int grid = (int)std::min<long long>(p.n_units, resident);
    void* args[] = {&p};
    if (cudaLaunchKernel(ent.func, dim3(grid), dim3(kThreads), args, ent.smem, stream) != cudaSuccess)
        return TOED_ERR_CUDA;
    if (launch_finalize(p, stream) != cudaSuccess) return TOED_ERR_CUDA;
    return TOED_OK;
}
