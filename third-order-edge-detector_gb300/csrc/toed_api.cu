// toed_api.cu -- host implementation of the C ABI declared in
// include/toed_gb300.h: argument checks, tap generation, the per-device
// scratch owned by a context, strip planning and kernel launches.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <cudaTypedefs.h>
#include <nvtx3/nvToolsExt.h>

#include "toed_common.cuh"
#include "toed_internal.h"

namespace toed {
DetectEntry detect_entry_r1(bool, bool, bool);
DetectEntry detect_entry_r2(bool, bool, bool);
DetectEntry detect_entry_r3(bool, bool, bool);
DetectEntry detect_entry_r4(bool, bool, bool);
DetectEntry detect_entry_r5(bool, bool, bool);
DetectEntry detect_entry_r6(bool, bool, bool);
DetectEntry detect_entry_r7(bool, bool, bool);
DetectEntry detect_entry_r8(bool, bool, bool);
DetectEntry detect_entry_r9(bool, bool, bool);
DetectEntry detect_entry_r10(bool, bool, bool);
DetectEntry detect_entry_r11(bool, bool, bool);
DetectEntry detect_entry_r12(bool, bool, bool);

DetectEntry detect_entry(int r, bool hyb, bool async, bool nmsto)
{
    if (nmsto) async = false;
    switch (r) {
    case 1: return detect_entry_r1(hyb, async, nmsto);
    case 2: return detect_entry_r2(hyb, async, nmsto);
    case 3: return detect_entry_r3(hyb, async, nmsto);
    case 4: return detect_entry_r4(hyb, async, nmsto);
    case 5: return detect_entry_r5(hyb, async, nmsto);
    case 6: return detect_entry_r6(hyb, async, nmsto);
    case 7: return detect_entry_r7(hyb, async, nmsto);
    case 8: return detect_entry_r8(hyb, async, nmsto);
    case 9: return detect_entry_r9(hyb, async, nmsto);
    case 10: return detect_entry_r10(hyb, async, nmsto);
    case 11: return detect_entry_r11(hyb, async, nmsto);
    case 12: return detect_entry_r12(hyb, async, nmsto);
    default: return DetectEntry{nullptr, 0};
    }
}

// Taps from the reference's own commented generator (cpu_toed.cpp:141-162),
// evaluated in double and rounded once to float.
void make_taps64(double sigma, int r, TapBlock64* tb)
{
    std::memset(tb, 0, sizeof(*tb));
    const double nrm = std::sqrt(2.0 * 3.14159265358979323846);
    const double s = sigma;
    for (int sh = 0; sh < 2; ++sh) {
        const double d = sh ? 0.5 : 0.0;
        for (int k = 0; k < 2 * r + 3; ++k) {
            const double x = (double)(k - (r + 1)) + d;
            const double e = std::exp(-(x * x) / (2.0 * s * s));
            tb->v[4 * sh + 0][k] = e / (nrm * s);
            tb->v[4 * sh + 1][k] = (-x * e) / (nrm * s * s * s);
            tb->v[4 * sh + 2][k] = ((x * x - s * s) * e) / (nrm * s * s * s * s * s);
            tb->v[4 * sh + 3][k] = ((x * (3.0 * s * s - x * x)) * e) / (nrm * s * s * s * s * s * s * s);
        }
    }
}

void make_taps(double sigma, int r, TapBlock* tb)
{
    TapBlock64 d;
    make_taps64(sigma, r, &d);
    for (int f = 0; f < 8; ++f)
        for (int k = 0; k < kMaxTaps; ++k) tb->v[f][k] = (float)d.v[f][k];
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    });
    return fn;
}

void encode_rows_map(CUtensorMap* m, DetImage& d, int r)
{
    d.tma = 0;
    d.tma_align = 1;
    d.tma_boxw = 0;
    const int esz = (d.dtype == TOED_U8) ? 1 : 4;
    const int align = 16 / esz;
    const int nin = kExt + 2 * r + 2;
    const int boxw = (nin + align - 1 + align - 1) / align * align;
    auto fn = encode_fn();
    if (!fn || (reinterpret_cast<uintptr_t>(d.src) & 15u) != 0 || ((long long)d.pitch * esz) % 16 != 0 ||
        boxw * esz > kRawRowBytes)
        return;
    const cuuint64_t dims[2] = {(cuuint64_t)d.W, (cuuint64_t)d.H};
    const cuuint64_t strides[1] = {(cuuint64_t)d.pitch * esz};
    const cuuint32_t box[2] = {(cuuint32_t)boxw, (cuuint32_t)kStepRows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult res = fn(m, esz == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                            const_cast<void*>(d.src), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (res != CUDA_SUCCESS) return;
    d.tma = 1;
    d.tma_align = align;
    d.tma_boxw = boxw;
}

}  // namespace toed

using namespace toed;

// NVTX range over one phase of a call (the detection launch, the ordering
// pass, a copy group, ...): no cost unless a profiler is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

static thread_local std::string g_last_cuda_error;

#define TOED_CU(call)                                                                 \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            g_last_cuda_error = std::string(#call) + ": " + cudaGetErrorString(e_);   \
            return TOED_ERR_CUDA;                                                     \
        }                                                                             \
    } while (0)

struct toed_ctx {
    int device = 0;
    int num_sms = 0;
    int* words = nullptr;  // kWords: [0] queue [1] cursor [2] flags [3] refine-list length [4] debug
    double4_32a* staging = nullptr;
    int* staging_idx = nullptr;
    long long staging_cap = 0;
    int2* seg = nullptr;
    long long seg_cap = 0;
    int* tile_sum = nullptr;
    long long tile_cap = 0;
    long long* img_base = nullptr;
    int img_cap = 0;
    int4* refine = nullptr;  // orientation recomputation list
    long long refine_cap = 0;
    float2* dir = nullptr;
    int* eid = nullptr;
    int* win = nullptr;
    long long px_cap = 0, px_cap2 = 0, px_cap3 = 0;
    int* img_count = nullptr;
    long long img_count_cap = 0;
    unsigned char* keep = nullptr;
    long long keep_cap = 0;
    double* sp_work = nullptr;  // TO correction at interp_n > 0: maps resized onto the work grid
    long long sp_work_cap = 0;
    int blocks_per_sm[TOED_MAX_RADIUS + 1][2][3] = {};  // [radius][hybrid][TMA/plain, async, corrected normal]
    // launch shape chosen by toed_autotune per (radius, precision, size class of
    // the launch: floor(log2(pixels))); strip_rows 0 = heuristic
    toed_tuning tune[TOED_MAX_RADIUS + 1][2][kSizeClasses] = {};
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof;
    // toed_detect_host_batch: device staging of images / lists / counts, a
    // page-locked count buffer and the copy streams
    unsigned char* hb_in = nullptr;
    long long hb_in_cap = 0;
    unsigned char* hb_out = nullptr;
    long long hb_out_cap = 0;
    int* hb_idx = nullptr;
    long long hb_idx_cap = 0;
    int* hb_cnt = nullptr;
    long long hb_cnt_cap = 0;
    int* hb_cnt_host = nullptr;
    long long hb_cnt_host_cap = 0;
    cudaStream_t s_in = nullptr, s_out = nullptr;
    // copy-group ready flags (device), the epoch they are set to (page-locked
    // source of the flag copies) and the epoch of the current call
    int* hb_ready = nullptr;
    long long hb_ready_cap = 0;
    int* hb_epoch_src = nullptr;
    int hb_epoch = 0;
    int ready_spins = kReadySpinLimit;  // bound of each ready-flag wait (polls)
    std::vector<cudaEvent_t> hb_ev;     // toed_detect_host_batch's ordering events, reused
    float tap_sigma = -1.f;             // taps of the last detection's (sigma, radius)
    int tap_r = 0;
    TapBlock taps;
    TapBlock64 taps64;
    std::mutex mu;
};

extern "C" {

void toed_params_default(toed_params* p, float sigma)
{
    if (!p) return;
    p->sigma = sigma;
    p->radius = 0;
    p->threshold = 2.0f;
    p->border = 10;
    p->out_dtype = TOED_F32;
    p->precision = TOED_HYBRID;
    p->orientation = TOED_ORI_GRID;
    p->nms_direction = TOED_NMS_GRADIENT;
}

const char* toed_status_string(toed_status s)
{
    switch (s) {
    case TOED_OK: return "ok";
    case TOED_ERR_INVALID_ARG: return "invalid argument";
    case TOED_ERR_CAPACITY: return "capacity exceeded";
    case TOED_ERR_CUDA: return "CUDA error";
    case TOED_ERR_TIMEOUT: return "device wait timed out";
    case TOED_ERR_UNSUPPORTED: return "unsupported configuration";
    case TOED_ERR_CAPTURE: return "scratch must grow during stream capture (call toed_reserve first)";
    }
    return "unknown status";
}

const char* toed_last_cuda_error(void) { return g_last_cuda_error.c_str(); }

toed_status toed_create(toed_ctx** out, int device)
{
    if (!out) return TOED_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    TOED_CU(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return TOED_ERR_INVALID_ARG;
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    TOED_CU(cudaSetDevice(device));
    toed_ctx* c = new toed_ctx();
    c->device = device;
    cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&c->words, kWords * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->words, 0, kWords * sizeof(int));
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        g_last_cuda_error = cudaGetErrorString(e);
        delete c;
        return TOED_ERR_CUDA;
    }
    *out = c;
    return TOED_OK;
}

toed_status toed_destroy(toed_ctx* c)
{
    if (!c) return TOED_ERR_INVALID_ARG;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(c->device);
    cudaFree(c->words);
    cudaFree(c->staging);
    cudaFree(c->staging_idx);
    cudaFree(c->seg);
    cudaFree(c->tile_sum);
    cudaFree(c->img_base);
    cudaFree(c->refine);
    cudaFree(c->dir);
    cudaFree(c->eid);
    cudaFree(c->win);
    cudaFree(c->img_count);
    cudaFree(c->keep);
    cudaFree(c->sp_work);
    cudaFree(c->hb_in);
    cudaFree(c->hb_out);
    cudaFree(c->hb_idx);
    cudaFree(c->hb_cnt);
    if (c->hb_cnt_host) cudaFreeHost(c->hb_cnt_host);
    if (c->hb_epoch_src) cudaFreeHost(c->hb_epoch_src);
    cudaFree(c->hb_ready);
    for (auto e : c->hb_ev) cudaEventDestroy(e);
    if (c->s_in) cudaStreamDestroy(c->s_in);
    if (c->s_out) cudaStreamDestroy(c->s_out);
    cudaSetDevice(prev);
    delete c;
    return TOED_OK;
}

}  // extern "C"

// Grow a device buffer; refuses while the stream is being captured.
template <typename T>
static toed_status grow(T** buf, long long* cap, long long need, cudaStream_t stream)
{
    if (need <= *cap) return TOED_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (stream) cudaStreamIsCapturing(stream, &cs);
    if (cs != cudaStreamCaptureStatusNone) return TOED_ERR_CAPTURE;
    long long n = std::max(need, *cap + *cap / 2);
    if (*buf) TOED_CU(cudaFree(*buf));
    *buf = nullptr;
    *cap = 0;
    TOED_CU(cudaMalloc((void**)buf, sizeof(T) * (size_t)n));
    *cap = n;
    return TOED_OK;
}

static toed_status ensure_scratch(toed_ctx* c, long long staging, long long segs, long long tiles,
                                  int imgs, cudaStream_t stream)
{
    toed_status st;
    long long sc = c->staging_cap;
    if ((st = grow(&c->staging, &sc, staging, stream)) != TOED_OK) return st;
    long long sc2 = c->staging_cap;
    if ((st = grow(&c->staging_idx, &sc2, staging, stream)) != TOED_OK) return st;
    c->staging_cap = std::min(sc, sc2);
    // one entry per 64 staged edgels (about 1 in 5000 is listed on noisy images)
    if ((st = grow(&c->refine, &c->refine_cap, staging / 64 + 1024, stream)) != TOED_OK) return st;
    if ((st = grow(&c->seg, &c->seg_cap, segs, stream)) != TOED_OK) return st;
    if ((st = grow(&c->tile_sum, &c->tile_cap, tiles, stream)) != TOED_OK) return st;
    long long ic = c->img_cap;
    if ((st = grow(&c->img_base, &ic, (long long)imgs, stream)) != TOED_OK) return st;
    c->img_cap = (int)ic;
    return TOED_OK;
}

extern "C" toed_status toed_reserve(toed_ctx* c, long long max_pixels, long long max_edgels, int max_images)
{
    if (!c || max_pixels < 0 || max_edgels < 0 || max_images < 0) return TOED_ERR_INVALID_ARG;
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    TOED_CU(cudaSetDevice(c->device));
    // segments: 2 rows per pixel row x ceil(W/30) strip columns, bounded by pixels/15 + tiles of padding
    const int imgs = std::min(std::max(max_images, 1), kBatchMax);
    const long long segs = max_pixels / 15 + 2LL * 4096 + (long long)imgs * kSegTile;
    const long long tiles = segs / kSegTile + imgs + 1;
    std::lock_guard<std::mutex> lk(c->mu);
    // staging slack: one reservation block per resident CTA (at most 4 per SM)
    const long long slack = 4LL * c->num_sms * kStageBlk;
    toed_status st = ensure_scratch(c, std::max(max_edgels, 1LL) + slack, segs, tiles, imgs, nullptr);
    cudaSetDevice(prev);
    return st;
}

toed_status toed::check_image(const toed_image& im)
{
    if (!im.pixels || !im.edgels || !im.count) return TOED_ERR_INVALID_ARG;
    if (im.height <= 0 || im.width <= 0 || im.pitch < im.width || im.capacity < 0) return TOED_ERR_INVALID_ARG;
    if (im.dtype != TOED_U8 && im.dtype != TOED_F32) return TOED_ERR_UNSUPPORTED;
    if ((long long)(2LL * im.height) * (2LL * im.width) >= (1LL << 31)) return TOED_ERR_UNSUPPORTED;
    if ((reinterpret_cast<uintptr_t>(im.edgels) & 15u) != 0) return TOED_ERR_INVALID_ARG;
    if (im.dtype == TOED_F32 && (reinterpret_cast<uintptr_t>(im.pixels) & 3u) != 0) return TOED_ERR_INVALID_ARG;
    return TOED_OK;
}

static int radius_of(const toed_params* p)
{
    if (p->radius > 0) return p->radius;
    return (int)std::ceil(4.0 * (double)p->sigma);
}

// Size class of one launch: floor(log2(pixels)).  A launch shape that wins
// on a 64-image batch is a poor one for a single small image, so tuned shapes
// are kept per class.
static int size_class(const toed_image* images, int n)
{
    long long px = 1;
    for (int i = 0; i < n; ++i) px += (long long)images[i].width * images[i].height;
    int k = 0;
    while (k + 1 < kSizeClasses && (px >> (k + 1)) > 0) ++k;
    return k;
}

// Strip height: the tallest multiple of the step (minus the 2-row ring) that
// still gives every resident CTA several units to balance the queue.
static int plan_strip_rows(const toed_image* images, int n, long long resident)
{
    static const int steps[] = {64, 32, 16, 8, 4, 2, 1};
    for (int st : steps) {
        const int S = st * kStepRows - 2;
        long long units = 0;
        for (int i = 0; i < n; ++i)
            units += (long long)((images[i].width + kInner - 1) / kInner) * ((images[i].height + S - 1) / S);
        if (units >= 4 * resident) return S;
    }
    return kStepRows - 2;
}

// plain_loads: never stage input rows by TMA (images read in place from
// page-locked host memory through their device mapping): float32 rows by
// per-thread async copies one step ahead, uint8 rows by plain loads
// wait_slot (optional, per image): 0, or g > 0 when the copy engine is still
// bringing the image in and c->hb_ready[g - 1] == c->hb_epoch marks its arrival
static toed_status detect_chunk(toed_ctx* c, const toed_image* images, int n, const toed_params* prm,
                                int r, bool first_chunk, cudaStream_t stream, const toed_tuning* force = nullptr,
                                bool plain_loads = false, const int* wait_slot = nullptr)
{
    const bool hyb = prm->precision != TOED_FP32;
    const bool nmsto = prm->nms_direction == TOED_NMS_TO_NORMAL;
    const toed_tuning& tuned = c->tune[r][hyb ? 1 : 0][size_class(images, n)];
    const toed_tuning* use = force ? force : (tuned.strip_rows > 0 ? &tuned : nullptr);
    // async row staging: images read in place from host memory, or the tuned
    // shape asks for it (the corrected-normal kernel stages rows by TMA or
    // plain loads only)
    const bool async_rows = !nmsto && (plain_loads || (use && use->staging == 2));
    DetectEntry ent = detect_entry(r, hyb, async_rows, nmsto);
    if (!ent.func) return TOED_ERR_UNSUPPORTED;
    int& bps = c->blocks_per_sm[r][hyb ? 1 : 0][nmsto ? 2 : (async_rows ? 1 : 0)];
    if (bps == 0) {
        TOED_CU(cudaFuncSetAttribute(ent.func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ent.smem));
        TOED_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ent.func, kThreads, ent.smem));
        if (bps <= 0) return TOED_ERR_UNSUPPORTED;
    }
    const long long resident = (long long)bps * c->num_sms;

    BatchParams* p = new BatchParams();
    std::unique_ptr<BatchParams> guard(p);
    // the taps of the last (sigma, radius), kept in the context (a few hundred exp per call otherwise)
    if (c->tap_sigma != prm->sigma || c->tap_r != r) {
        make_taps((double)prm->sigma, r, &c->taps);
        make_taps64((double)prm->sigma, r, &c->taps64);
        c->tap_sigma = prm->sigma;
        c->tap_r = r;
    }
    p->taps = c->taps;
    p->taps64 = c->taps64;
    p->thr = prm->threshold;
    p->thr2 = prm->threshold < 0.f ? -1.f : prm->threshold * prm->threshold * 0.9999f;
    p->border = prm->border;
    p->S = use ? use->strip_rows : plan_strip_rows(images, n, resident);
    p->n_img = n;
    p->out_f64 = (prm->out_dtype == TOED_F64) ? 1 : 0;
    p->radius = r;
    p->hyb = hyb ? 1 : 0;
    p->qad = prm->orientation == TOED_ORI_QAD ? 1 : 0;
    p->nms_to = nmsto ? 1 : 0;
    p->det_rec = 1;
    p->ready = c->hb_ready;
    p->ready_epoch = c->hb_epoch;
    p->ready_spins = c->ready_spins;
    // A work unit at the tuned shape can take several percent of the launch
    // (a 1022-row unit about 260 us of a 2.2 ms batch), and as the queue
    // drains the last units leave SMs idle while they run.  So an image's
    // strips are halved (64 steps of 16 rows -> 32 -> ... -> 2, i.e. 1022
    // -> 510 -> ... -> 30 rows) until the pixels from its start to the end
    // of the batch hold at least one of its units per resident CTA: the
    // launch ends with small units.  (Measured on a 64-image batch: 2.155 ms,
    // against 2.158 with two units per CTA, 2.182 with four and 2.221
    // without.  A single image keeps the tuned strips, which the tuner picks
    // for its size alone.)
    long long npx = 0, cum = 0;
    for (int i = 0; i < n; ++i) npx += (long long)images[i].width * images[i].height;
    long long units = 0, tiles = 0, staging = 0;
    for (int i = 0; i < n; ++i) {
        const toed_image& im = images[i];
        DetImage& d = p->img[i];
        int ksteps = (p->S + 2) / kStepRows;  // steps per strip
        while (n > 1 && ksteps > 2 && (long long)(ksteps * kStepRows - 2) * kInner * resident > npx - cum)
            ksteps = std::max(2, ksteps / 2);
        d.S = ksteps * kStepRows - 2;
        cum += (long long)im.width * im.height;
        d.src = im.pixels;
        d.pitch = im.pitch;
        d.out = im.edgels;
        d.count = im.count;
        d.index = im.grid_index;
        d.H = im.height;
        d.W = im.width;
        d.dtype = im.dtype;
        d.cap = im.capacity;
        d.nsc = (im.width + kInner - 1) / kInner;
        d.nsr = (im.height + d.S - 1) / d.S;
        d.unit_base = (int)units;
        d.tile_base = (int)tiles;
        d.seg_base = tiles * kSegTile;
        d.wait_slot = wait_slot ? wait_slot[i] : 0;
        d.tma_align = 1;
        d.tma_boxw = 0;
        if (async_rows)
            d.tma = (d.dtype == TOED_F32) ? 2 : 0;  // async row copies (float32) or plain loads, never TMA
        else if ((use && !use->staging) || plain_loads)
            d.tma = 0;  // plain loads (host memory read in place: never TMA)
        else
            encode_rows_map(&p->tmap[i], d, r);  // TMA where the image allows it (a host call per image)
        const long long nseg = 2LL * im.height * d.nsc;
        d.nseg = nseg;
        units += (long long)d.nsc * d.nsr;
        tiles += (nseg + kSegTile - 1) / kSegTile;
        staging += im.capacity;
    }
    if (units >= (1LL << 31) || tiles >= (1LL << 31)) return TOED_ERR_UNSUPPORTED;
    p->n_units = (int)units;
    p->n_tiles = (int)tiles;
    // every resident CTA may leave up to one reservation block of staging unused
    p->stage_blk = kStageBlk;
    staging += resident * kStageBlk;
    toed_status st = ensure_scratch(c, std::max(staging, 1LL), tiles * kSegTile, tiles, n, stream);
    if (st != TOED_OK) return st;
    p->sc.words = c->words;
    p->sc.staging = c->staging;
    p->sc.staging_idx = c->staging_idx;
    p->sc.staging_cap = c->staging_cap;
    p->sc.seg = c->seg;
    p->sc.seg_cap = c->seg_cap;
    p->sc.tile_sum = c->tile_sum;
    p->sc.img_base = c->img_base;
    // FP64 orientation recomputation: hybrid precision, grid orientation
    // (the subpixel orientation replaces the staged one)
    p->sc.refine = c->refine;
    p->sc.refine_cap = (hyb && !p->qad) ? (int)std::min<long long>(c->refine_cap, 1LL << 30) : 0;

    // the first chunk clears the flags and the refine-list length too; later
    // chunks find the list emptied by the previous ordering pass
    TOED_CU(cudaMemsetAsync(c->words, 0, (first_chunk ? kWords : 2) * sizeof(int), stream));
    const int grid = (int)std::min<long long>(units, resident);
    void* args[] = {p};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (c->profiling) {
        TOED_CU(cudaEventCreate(&ev0));
        TOED_CU(cudaEventCreate(&ev1));
        c->prof.emplace_back(ev0, ev1);
        TOED_CU(cudaEventRecord(ev0, stream));
    }
    {
        NvtxRange r("toed: detection launch");
        TOED_CU(cudaLaunchKernel(ent.func, dim3(grid), dim3(kThreads), args, ent.smem, stream));
    }
    if (ev1) TOED_CU(cudaEventRecord(ev1, stream));
    {
        NvtxRange r("toed: ordering pass");
        TOED_CU(launch_finalize(*p, stream));
    }
    return TOED_OK;
}

static toed_status check_batch(const toed_ctx* c, const toed_image* images, int n, const toed_params* prm)
{
    if (!c || !images || n <= 0 || !prm) return TOED_ERR_INVALID_ARG;
    if (!(prm->sigma > 0.f) || !std::isfinite(prm->sigma) || !std::isfinite(prm->threshold)) return TOED_ERR_INVALID_ARG;
    if (prm->border < 1) return TOED_ERR_INVALID_ARG;
    if (prm->out_dtype != TOED_F32 && prm->out_dtype != TOED_F64) return TOED_ERR_INVALID_ARG;
    if (prm->precision != TOED_HYBRID && prm->precision != TOED_FP32) return TOED_ERR_INVALID_ARG;
    if (prm->orientation != TOED_ORI_GRID && prm->orientation != TOED_ORI_QAD) return TOED_ERR_INVALID_ARG;
    if (prm->nms_direction != TOED_NMS_GRADIENT && prm->nms_direction != TOED_NMS_TO_NORMAL)
        return TOED_ERR_INVALID_ARG;
    // the quick-and-dirty orientation is defined on the gradient-direction NMS
    if (prm->nms_direction == TOED_NMS_TO_NORMAL && prm->orientation != TOED_ORI_GRID) return TOED_ERR_UNSUPPORTED;
    const int r = radius_of(prm);
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    for (int i = 0; i < n; ++i) {
        toed_status st = check_image(images[i]);
        if (st != TOED_OK) return st;
    }
    return TOED_OK;
}

// The batch in chunks of kBatchMax images (caller holds c->mu, device set).
static toed_status detect_all(toed_ctx* c, const toed_image* images, int n, const toed_params* prm,
                              cudaStream_t stream, const toed_tuning* force = nullptr, bool plain_loads = false,
                              const int* wait_slot = nullptr)
{
    const int r = radius_of(prm);
    toed_status st = TOED_OK;
    for (int i0 = 0; i0 < n && st == TOED_OK; i0 += kBatchMax)
        st = detect_chunk(c, images + i0, std::min(kBatchMax, n - i0), prm, r, i0 == 0, stream, force, plain_loads,
                          wait_slot ? wait_slot + i0 : nullptr);
    return st;
}

extern "C" toed_status toed_detect_batch(toed_ctx* c, const toed_image* images, int n,
                                         const toed_params* prm, cudaStream_t stream)
{
    NvtxRange nv("toed_detect_batch");
    toed_status st = check_batch(c, images, n, prm);
    if (st != TOED_OK) return st;
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    if (prev != c->device) TOED_CU(cudaSetDevice(c->device));
    {
        std::lock_guard<std::mutex> lk(c->mu);
        st = detect_all(c, images, n, prm, stream);
    }
    if (prev != c->device) cudaSetDevice(prev);
    return st;
}

// Times every candidate launch shape on the caller's batch (CUDA events on
// its stream, after one untimed run each) and keeps the fastest.  The
// candidates change only how the work is cut and staged -- strip height and
// TMA vs plain row loads -- never the result, which is the same bit for bit.
extern "C" toed_status toed_autotune(toed_ctx* c, const toed_image* images, int n, const toed_params* prm,
                                     int reps, cudaStream_t stream, toed_tuning* best)
{
    NvtxRange nv("toed_autotune");
    toed_status st = check_batch(c, images, n, prm);
    if (st != TOED_OK) return st;
    if (reps < 1) return TOED_ERR_INVALID_ARG;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    TOED_CU(cudaStreamIsCapturing(stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) return TOED_ERR_CAPTURE;
    const int r = radius_of(prm);
    const int hyb = prm->precision != TOED_FP32 ? 1 : 0;
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    if (prev != c->device) TOED_CU(cudaSetDevice(c->device));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    toed_tuning win = {};
    win.ms = -1.f;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        cudaError_t ce = cudaEventCreate(&e0);
        if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
        if (ce != cudaSuccess) {
            g_last_cuda_error = std::string("autotune: ") + cudaGetErrorString(ce);
            st = TOED_ERR_CUDA;
        }
        // strip heights of 1..64 steps: powers of two and the steps between
        // them (a small image's best height fills the resident CTAs once)
        static const int steps[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64};
        constexpr int kCand = (int)(sizeof(steps) / sizeof(steps[0]));
        for (int staging = 2; staging >= 0 && st == TOED_OK; --staging)
            for (int k = 0; k < kCand && st == TOED_OK; ++k) {
                toed_tuning cand = {steps[k] * kStepRows - 2, staging, 0.f};
                st = detect_all(c, images, n, prm, stream, &cand);  // untimed: scratch, caches
                if (st != TOED_OK) break;
                ce = cudaEventRecord(e0, stream);
                for (int i = 0; i < reps && st == TOED_OK && ce == cudaSuccess; ++i)
                    st = detect_all(c, images, n, prm, stream, &cand);
                if (ce == cudaSuccess) ce = cudaEventRecord(e1, stream);
                if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
                if (ce != cudaSuccess) {
                    g_last_cuda_error = std::string("autotune: ") + cudaGetErrorString(ce);
                    st = TOED_ERR_CUDA;
                    break;
                }
                cand.ms = ms / (float)reps;
                if (st == TOED_OK && (win.ms < 0.f || cand.ms < win.ms)) win = cand;
            }
        if (st == TOED_OK)
            for (int i0 = 0; i0 < n; i0 += kBatchMax)
                c->tune[r][hyb][size_class(images + i0, std::min(kBatchMax, n - i0))] = win;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (prev != c->device) cudaSetDevice(prev);
    if (st == TOED_OK && best) *best = win;
    return st;
}

extern "C" toed_status toed_set_tuning(toed_ctx* c, const toed_params* prm, const toed_tuning* t)
{
    if (!c || !prm) return TOED_ERR_INVALID_ARG;
    const int r = radius_of(prm);
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    toed_tuning v = {};
    if (t) {
        if (t->strip_rows < kStepRows - 2 || (t->strip_rows + 2) % kStepRows != 0 || t->strip_rows > 64 * kStepRows - 2 ||
            (t->staging < 0 || t->staging > 2))
            return TOED_ERR_INVALID_ARG;
        v = *t;
    }
    std::lock_guard<std::mutex> lk(c->mu);
    for (int k = 0; k < kSizeClasses; ++k) c->tune[r][prm->precision != TOED_FP32 ? 1 : 0][k] = v;
    return TOED_OK;
}

extern "C" toed_status toed_detect(toed_ctx* c, const toed_image* image, const toed_params* prm,
                                   cudaStream_t stream)
{
    return toed_detect_batch(c, image, 1, prm, stream);
}

// Launches run one at a time, each waited for: CUDA_LAUNCH_BLOCKING=1, or a
// tool injected into the runtime (profilers and checkers serialise work).
// (Nsight Compute marks its target process with NV_NSIGHT_INJECTION_* and
// NV_COMPUTE_PROFILER_PERFWORKS_DIR; runtime-injected tools with
// CUDA_INJECTION64_PATH.)
static bool launches_serialised()
{
    const char* lb = std::getenv("CUDA_LAUNCH_BLOCKING");
    if (lb && lb[0] == '1') return true;
    for (const char* v : {"CUDA_INJECTION64_PATH", "NV_NSIGHT_INJECTION_TRANSPORT_TYPE",
                          "NV_COMPUTE_PROFILER_PERFWORKS_DIR"}) {
        const char* e = std::getenv(v);
        if (e && e[0]) return true;
    }
    return false;
}

// Host-memory batch, pipelined over `chunks` groups of images (see the
// header).  Streams: s_in (H2D), the caller's stream (detection), s_out
// (D2H, pageable outputs only); events order them per group.
extern "C" toed_status toed_detect_host_batch(toed_ctx* c, const toed_host_image* images, int n,
                                              const toed_params* prm, int chunks, cudaStream_t stream)
{
    NvtxRange nv("toed_detect_host_batch");
    if (!c || !images || n <= 0 || !prm) return TOED_ERR_INVALID_ARG;
    std::vector<toed_image> dev(n);
    std::vector<long long> in_off(n), out_off(n), idx_off(n);
    const int rec = prm->out_dtype == TOED_F64 ? 32 : 16;
    long long in_b = 0, out_b = 0, idx_n = 0, total_px = 0;
    for (int i = 0; i < n; ++i) {
        const toed_host_image& h = images[i];
        if (!h.pixels || !h.edgels || !h.count || h.height <= 0 || h.width <= 0 || h.pitch < h.width ||
            h.capacity < 0)
            return TOED_ERR_INVALID_ARG;
        if (h.dtype != TOED_U8 && h.dtype != TOED_F32) return TOED_ERR_UNSUPPORTED;
        const int esz = h.dtype == TOED_U8 ? 1 : 4;
        const long long dpitch = ((long long)h.width * esz + 15) / 16 * 16;  // 16-byte rows: TMA-eligible
        in_off[i] = in_b;
        in_b += (dpitch * h.height + 255) / 256 * 256;
        out_off[i] = out_b;
        out_b += ((long long)std::max(h.capacity, 1) * rec + 255) / 256 * 256;
        idx_off[i] = idx_n;
        if (h.grid_index) idx_n += std::max(h.capacity, 1);
        total_px += (long long)h.height * h.width;
        dev[i].height = h.height;
        dev[i].width = h.width;
        dev[i].pitch = (int)(dpitch / esz);
        dev[i].dtype = h.dtype;
        dev[i].capacity = h.capacity;
    }
    chunks = std::max(1, std::min(chunks, n));
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    TOED_CU(cudaStreamIsCapturing(stream, &cs));
    if (cs != cudaStreamCaptureStatusNone) return TOED_ERR_CAPTURE;
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    if (prev != c->device) TOED_CU(cudaSetDevice(c->device));
    std::lock_guard<std::mutex> lk(c->mu);
    toed_status st = TOED_OK;
    std::vector<cudaEvent_t> ev_in(chunks, nullptr), ev_det(chunks, nullptr);
    std::vector<int> first(chunks + 1, n);
    auto fail = [&](toed_status s) {
        // an early return must not leave copies in flight: the next call
        // reuses the staging and rewrites the epoch their flag copies read
        if (s != TOED_OK && c->s_in) cudaStreamSynchronize(c->s_in);
        if (prev != c->device) cudaSetDevice(prev);
        return s;
    };
#define TOED_HB(call)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            g_last_cuda_error = std::string(#call) + ": " + cudaGetErrorString(e_);       \
            return fail(TOED_ERR_CUDA);                                                   \
        }                                                                                 \
    } while (0)
    // Page-locked host outputs are written by the ordering pass itself
    // (mapped into the device's address space; coherent over the C2C link):
    // no count read-back and no list copies.  Otherwise lists go through
    // device staging and are copied back per group once its counts are known.
    auto mapped = [](void* hp) -> void* {
        cudaPointerAttributes a;
        if (!hp || cudaPointerGetAttributes(&a, hp) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
    };
    // Page-locked inputs: with chunks == 1 the detection kernel reads them in
    // place through their device mapping (zero copy over the C2C link); with
    // more groups the copy engine brings the groups into device memory while
    // ONE detection launch runs, each image's CTAs waiting (bounded) for its
    // group's ready flag, which the copy engine writes after the group's
    // pixels -- every pixel crosses the link once and no group boundary
    // drains the GPU.  Pageable inputs: staged copies per group, one
    // detection launch per group once its copy is in.
    bool zin = true;
    std::vector<const void*> in_map(n, nullptr);
    for (int i = 0; i < n && zin; ++i) {
        in_map[i] = mapped(const_cast<void*>(images[i].pixels));
        zin = in_map[i] != nullptr;
    }
    // (flagged: one launch of at most kBatchMax images, so that nothing between
    // the launch and the copies' enqueueing can wait for the device; never
    // when launches run serialised -- CUDA_LAUNCH_BLOCKING, or a profiler or
    // checker injected into the runtime -- since then the waiting launch
    // would hold the host or the device until its wait gives up)
    const bool inplace = zin && chunks == 1,
               flagged = zin && chunks > 1 && n <= kBatchMax && !launches_serialised();
    if (!inplace && (st = grow(&c->hb_in, &c->hb_in_cap, std::max(in_b, 1LL), stream)) != TOED_OK) return fail(st);
    if (flagged) {
        const long long had = c->hb_ready_cap;
        if ((st = grow(&c->hb_ready, &c->hb_ready_cap, (long long)chunks, stream)) != TOED_OK) return fail(st);
        if (c->hb_ready_cap != had) TOED_HB(cudaMemsetAsync(c->hb_ready, 0, sizeof(int) * c->hb_ready_cap, stream));
        if (!c->hb_epoch_src) TOED_HB(cudaMallocHost((void**)&c->hb_epoch_src, sizeof(int)));
        // a new epoch per call: flags left by earlier calls never match
        c->hb_epoch = c->hb_epoch % 0x3fffffff + 1;
        *c->hb_epoch_src = c->hb_epoch;
    }
    if ((st = grow(&c->hb_out, &c->hb_out_cap, std::max(out_b, 1LL), stream)) != TOED_OK) return fail(st);
    if ((st = grow(&c->hb_idx, &c->hb_idx_cap, std::max(idx_n, 1LL), stream)) != TOED_OK) return fail(st);
    if ((st = grow(&c->hb_cnt, &c->hb_cnt_cap, (long long)n + chunks, stream)) != TOED_OK) return fail(st);
    if (c->hb_cnt_host_cap < (long long)n + chunks) {
        if (c->hb_cnt_host) cudaFreeHost(c->hb_cnt_host);
        c->hb_cnt_host = nullptr;
        c->hb_cnt_host_cap = 0;
        TOED_HB(cudaMallocHost((void**)&c->hb_cnt_host, sizeof(int) * (size_t)(n + chunks)));
        c->hb_cnt_host_cap = n + chunks;
    }
    if (!c->s_in) TOED_HB(cudaStreamCreateWithFlags(&c->s_in, cudaStreamNonBlocking));
    if (!c->s_out) TOED_HB(cudaStreamCreateWithFlags(&c->s_out, cudaStreamNonBlocking));
    bool direct = true;
    for (int i = 0; i < n && direct; ++i) {
        void* e = mapped(images[i].edgels);
        void* cn = mapped(images[i].count);
        void* gi = images[i].grid_index ? mapped(images[i].grid_index) : nullptr;
        direct = e && cn && (!images[i].grid_index || gi);
        dev[i].edgels = e;
        dev[i].count = static_cast<int*>(cn);
        dev[i].grid_index = static_cast<int*>(gi);
    }
    for (int i = 0; i < n; ++i) {
        dev[i].pixels = inplace ? in_map[i] : c->hb_in + in_off[i];
        if (inplace) dev[i].pitch = images[i].pitch;
        if (!direct) {
            dev[i].edgels = c->hb_out + out_off[i];
            dev[i].count = c->hb_cnt + i;
            dev[i].grid_index = images[i].grid_index ? c->hb_idx + idx_off[i] : nullptr;
        }
    }
    for (int i = 0; i < n; ++i) {
        st = check_image(dev[i]);
        if (st != TOED_OK) return fail(st);
    }
    // groups of consecutive images whose pixel counts grow geometrically
    // (ratio at most detection time / copy time per pixel, about 1.6): the
    // first group is small so detection starts early, and each later copy
    // still finishes before the detection in front of it.  Flagged groups
    // cost no launch, so they grow more slowly (1.3) from a smaller start.
    {
        const double g = flagged ? 1.3 : 1.6, gn = std::pow(g, chunks) - 1.0;
        long long acc = 0;
        int k = 0;
        first[0] = 0;
        for (int i = 0; i < n && k + 1 < chunks; ++i) {
            acc += (long long)images[i].height * images[i].width;
            if ((double)acc >= (double)total_px * (std::pow(g, k + 1) - 1.0) / gn && i + 1 < n) first[++k] = i + 1;
        }
        chunks = k + 1;
        first[chunks] = n;
    }
    // the ordering events live in the context (the call is synchronous: none
    // is pending when the next call reuses it)
    while ((int)c->hb_ev.size() < 2 * chunks) {
        cudaEvent_t e = nullptr;
        TOED_HB(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->hb_ev.push_back(e);
    }
    for (int k = 0; k < chunks; ++k) {
        ev_in[k] = c->hb_ev[2 * k];
        ev_det[k] = c->hb_ev[2 * k + 1];
    }
    auto copy_group = [&](int k) -> cudaError_t {  // group k's images to the device on s_in
        for (int i = first[k]; i < first[k + 1]; ++i) {
            const toed_host_image& h = images[i];
            const int esz = h.dtype == TOED_U8 ? 1 : 4;
            // whole-image 1-D copies where the rows are contiguous: those run on the copy engines
            const cudaError_t e =
                (h.pitch == h.width && dev[i].pitch == h.width)
                    ? cudaMemcpyAsync(const_cast<void*>(dev[i].pixels), h.pixels, (size_t)h.width * h.height * esz,
                                      cudaMemcpyHostToDevice, c->s_in)
                    : cudaMemcpy2DAsync(const_cast<void*>(dev[i].pixels), (size_t)dev[i].pitch * esz, h.pixels,
                                        (size_t)h.pitch * esz, (size_t)h.width * esz, (size_t)h.height,
                                        cudaMemcpyHostToDevice, c->s_in);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    // launch groups: the detection launches, each followed by a read of the flags word
    int launches = chunks;
    if (flagged) {
        // Host-side failure injection for tests (no device fault): with
        // TOED_TEST_WITHHOLD_READY=k the ready-flag copy of group k is not
        // enqueued, so that group's units wait TOED_TEST_READY_SPINS polls
        // (default: the normal bound), give up, and the call returns
        // TOED_ERR_TIMEOUT; the image copies themselves still run.
        int withhold = -1;
        if (const char* e = std::getenv("TOED_TEST_WITHHOLD_READY")) withhold = std::atoi(e);
        c->ready_spins = kReadySpinLimit;
        if (const char* e = std::getenv("TOED_TEST_READY_SPINS"))
            c->ready_spins = std::max(1, std::min(std::atoi(e), kReadySpinLimit));
        // the copies wait only for what the caller's stream held before this
        // call (never for the detection launch, whose CTAs wait for them)
        TOED_HB(cudaEventRecord(ev_in[0], stream));
        TOED_HB(cudaStreamWaitEvent(c->s_in, ev_in[0], 0));
        std::vector<int> slot(n);
        for (int k = 0; k < chunks; ++k)
            for (int i = first[k]; i < first[k + 1]; ++i) slot[i] = k + 1;
        auto enqueue_group = [&](int k) -> cudaError_t {  // group k's pixels, then its flag, on s_in
            NvtxRange r("toed: copy group");
            cudaError_t e = copy_group(k);
            if (e == cudaSuccess && k != withhold)
                e = cudaMemcpyAsync(c->hb_ready + k, c->hb_epoch_src, sizeof(int), cudaMemcpyHostToDevice, c->s_in);
            return e;
        };
        // the first two groups go in before the launch, so that their pixels
        // are crossing while it is set up (the copies never wait for the
        // launch, so nothing up to it can wait on the device for long)
        const int early = std::min(chunks, 2);
        for (int k = 0; k < early; ++k) TOED_HB(enqueue_group(k));
        TOED_HB(preload_finalize(radius_of(prm), prm->orientation == TOED_ORI_QAD));
        st = detect_all(c, dev.data(), n, prm, stream, nullptr, true, slot.data());
        c->ready_spins = kReadySpinLimit;
        if (st != TOED_OK) return fail(st);
        TOED_HB(cudaMemcpyAsync(c->hb_cnt + n, c->words + 2, sizeof(int), cudaMemcpyDeviceToDevice, stream));
        TOED_HB(cudaEventRecord(ev_det[0], stream));
        for (int k = early; k < chunks; ++k) TOED_HB(enqueue_group(k));
        launches = 1;
        first[1] = n;
    } else {
        // 1. every group's images to the device, in order
        for (int k = 0; k < chunks && !inplace; ++k) {
            TOED_HB(copy_group(k));
            TOED_HB(cudaEventRecord(ev_in[k], c->s_in));
        }
        // 2. detection of each group once its images are in
        for (int k = 0; k < chunks; ++k) {
            if (!inplace) TOED_HB(cudaStreamWaitEvent(stream, ev_in[k], 0));
            st = detect_all(c, dev.data() + first[k], first[k + 1] - first[k], prm, stream, nullptr, inplace);
            if (st != TOED_OK) return fail(st);
            TOED_HB(cudaMemcpyAsync(c->hb_cnt + n + k, c->words + 2, sizeof(int), cudaMemcpyDeviceToDevice, stream));
            TOED_HB(cudaEventRecord(ev_det[k], stream));
        }
    }
    // 3. per group: counts (and the group's device flags) to the host, then
    // the lists, while later groups are still being copied in or detected
    int flags = 0;
    NvtxRange wait_range("toed: wait for counts and lists");
    if (direct) {
        TOED_HB(cudaMemcpyAsync(c->hb_cnt_host + n, c->hb_cnt + n, sizeof(int) * launches, cudaMemcpyDeviceToHost,
                                stream));
        TOED_HB(cudaStreamSynchronize(stream));
        for (int k = 0; k < launches; ++k) flags |= c->hb_cnt_host[n + k];
    }
    for (int k = 0; k < launches && !direct; ++k) {
        TOED_HB(cudaStreamWaitEvent(c->s_out, ev_det[k], 0));
        const int i0 = first[k], nk = first[k + 1] - first[k];
        TOED_HB(cudaMemcpyAsync(c->hb_cnt_host + i0, c->hb_cnt + i0, sizeof(int) * nk, cudaMemcpyDeviceToHost,
                                c->s_out));
        TOED_HB(cudaMemcpyAsync(c->hb_cnt_host + n + k, c->hb_cnt + n + k, sizeof(int), cudaMemcpyDeviceToHost,
                                c->s_out));
        TOED_HB(cudaStreamSynchronize(c->s_out));
        flags |= c->hb_cnt_host[n + k];
        for (int i = i0; i < i0 + nk; ++i) {
            const toed_host_image& h = images[i];
            const int cnt = c->hb_cnt_host[i];
            *h.count = cnt;
            const long long m = std::min(cnt, h.capacity);
            if (m <= 0) continue;
            TOED_HB(cudaMemcpyAsync(h.edgels, dev[i].edgels, (size_t)m * rec, cudaMemcpyDeviceToHost, c->s_out));
            if (h.grid_index)
                TOED_HB(cudaMemcpyAsync(h.grid_index, dev[i].grid_index, sizeof(int) * (size_t)m,
                                        cudaMemcpyDeviceToHost, c->s_out));
        }
    }
    TOED_HB(cudaStreamSynchronize(c->s_out));
    TOED_HB(cudaStreamSynchronize(stream));
    TOED_HB(cudaStreamSynchronize(c->s_in));
#undef TOED_HB
    fail(TOED_OK);  // releases the events, restores the device
    if (flags & TOED_FLAG_TIMEOUT) return TOED_ERR_TIMEOUT;
    if (flags & TOED_FLAG_STAGING_FULL) return TOED_ERR_CAPACITY;
    return TOED_OK;
}

extern "C" toed_status toed_device_flags(toed_ctx* c, cudaStream_t stream, int* flags)
{
    if (!c || !flags) return TOED_ERR_INVALID_ARG;
    int w[4] = {0, 0, 0, 0};
    TOED_CU(cudaMemcpyAsync(w, c->words, sizeof(w), cudaMemcpyDeviceToHost, stream));
    TOED_CU(cudaStreamSynchronize(stream));
    *flags = w[2];
    return TOED_OK;
}

extern "C" toed_status toed_profile_begin(toed_ctx* c)
{
    if (!c) return TOED_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    c->profiling = true;
    return TOED_OK;
}

extern "C" toed_status toed_profile_end(toed_ctx* c, double* kernel_ms, int* launches)
{
    if (!c || !kernel_ms || !launches) return TOED_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    c->profiling = false;
    double tot = 0.0;
    cudaError_t err = cudaSuccess;
    for (auto& pr : c->prof) {
        float ms = 0.f;
        if (err == cudaSuccess) err = cudaEventSynchronize(pr.second);
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, pr.first, pr.second);
        tot += ms;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    *launches = (int)c->prof.size();
    c->prof.clear();
    *kernel_ms = tot;
    if (err != cudaSuccess) {
        g_last_cuda_error = cudaGetErrorString(err);
        return TOED_ERR_CUDA;
    }
    return TOED_OK;
}

extern "C" toed_status toed_subpix_to_correct_batch(toed_ctx* c, const toed_edgemap* maps, int n,
                                                    const toed_subpix_params* prm, cudaStream_t stream)
{
    NvtxRange nv("toed_subpix_to_correct_batch");
    if (!c || !maps || n <= 0 || !prm) return TOED_ERR_INVALID_ARG;
    if (!(prm->sigma > 0.f) || !std::isfinite(prm->sigma) || !std::isfinite(prm->thresh) ||
        !std::isfinite(prm->nbr_radius))
        return TOED_ERR_INVALID_ARG;
    if (prm->out_dtype != TOED_F32 && prm->out_dtype != TOED_F64) return TOED_ERR_INVALID_ARG;
    if (prm->precision != TOED_HYBRID && prm->precision != TOED_FP32) return TOED_ERR_INVALID_ARG;
    if (prm->interp_n < 0 || prm->interp_n > 4) return TOED_ERR_INVALID_ARG;
    const int sc = 1 << prm->interp_n;  // work grid (h-1) sc + 1 by (w-1) sc + 1
    const int r = (int)std::ceil((double)prm->sigma * 4.0);  // build_gaussian_kernels radius
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    for (int i = 0; i < n; ++i) {
        const toed_edgemap& m = maps[i];
        if (!m.E || !m.edgels || !m.count || m.height < 2 || m.width < 2 || m.pitch < m.width || m.capacity < 0)
            return TOED_ERR_INVALID_ARG;
        if (m.dtype != TOED_F32 && m.dtype != TOED_F64) return TOED_ERR_UNSUPPORTED;
        if ((long long)((m.height - 1) * (long long)sc + 1) * ((m.width - 1) * (long long)sc + 1) >= (1LL << 31))
            return TOED_ERR_UNSUPPORTED;
        if ((reinterpret_cast<uintptr_t>(m.edgels) & 15u) != 0) return TOED_ERR_INVALID_ARG;
    }
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    if (prev != c->device) TOED_CU(cudaSetDevice(c->device));
    toed_status st = TOED_OK;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        for (int i0 = 0; i0 < n && st == TOED_OK; i0 += kBatchMax) {
            const int cn = std::min(kBatchMax, n - i0);
            const toed_edgemap* mp = maps + i0;
            long long px = 0, stag = 0, segs = 0, segtiles = 0, work = 0;
            for (int i = 0; i < cn; ++i) {
                const long long wh = (long long)(mp[i].height - 1) * sc + 1, ww = (long long)(mp[i].width - 1) * sc + 1;
                const long long hw = wh * ww;  // work-grid pixels
                px += hw;
                // every NMS edgel is staged before isolated ones are removed:
                // at most one per pixel, in practice far fewer than half
                stag += std::max<long long>(mp[i].capacity, hw / 2 + 1024);
                const long long nseg = wh * ((ww + 31) / 32);
                segtiles += (nseg + kSegTile - 1) / kSegTile;
                if (sc > 1) work += hw * (mp[i].theta ? 2 : 1);
            }
            segs = segtiles * kSegTile;
            if ((st = ensure_scratch(c, stag, segs, segtiles, cn, stream)) != TOED_OK) break;
            if ((st = grow(&c->dir, &c->px_cap, px, stream)) != TOED_OK) break;
            if ((st = grow(&c->eid, &c->px_cap2, px, stream)) != TOED_OK) break;
            if ((st = grow(&c->win, &c->px_cap3, px, stream)) != TOED_OK) break;
            if ((st = grow(&c->img_count, &c->img_count_cap, (long long)cn, stream)) != TOED_OK) break;
            if ((st = grow(&c->keep, &c->keep_cap, c->staging_cap, stream)) != TOED_OK) break;
            if (work > 0 && (st = grow(&c->sp_work, &c->sp_work_cap, work, stream)) != TOED_OK) break;
            SubScratch s;
            s.sc.words = c->words;
            s.sc.staging = c->staging;
            s.sc.staging_idx = c->staging_idx;
            s.sc.staging_cap = std::min(c->staging_cap, c->keep_cap);
            s.sc.seg = c->seg;
            s.sc.seg_cap = c->seg_cap;
            s.sc.tile_sum = c->tile_sum;
            s.sc.img_base = c->img_base;
            s.dir = c->dir;
            s.eid = c->eid;
            s.win = c->win;
            s.img_count = c->img_count;
            s.keep = c->keep;
            s.work = c->sp_work;
            cudaError_t e = subpix_launch(mp, cn, prm, r, s, stream);
            if (e != cudaSuccess) {
                g_last_cuda_error = std::string("subpix_launch: ") + cudaGetErrorString(e);
                st = TOED_ERR_CUDA;
            }
        }
    }
    if (prev != c->device) cudaSetDevice(prev);
    return st;
}

extern "C" toed_status toed_backward_batch(toed_ctx* c, const toed_grad_image* items, int n, const toed_params* prm,
                                           double* grad_sigma, cudaStream_t stream)
{
    NvtxRange nv("toed_backward_batch");
    if (!c || !items || n <= 0 || !prm || !grad_sigma) return TOED_ERR_INVALID_ARG;
    if (!(prm->sigma > 0.f) || !std::isfinite(prm->sigma)) return TOED_ERR_INVALID_ARG;
    // the adjoint is that of the grid-point orientation (cpu_toed.cpp:227-232)
    // and of the gradient-direction NMS (cpu_toed.cpp:411-489)
    if (prm->orientation != TOED_ORI_GRID || prm->nms_direction != TOED_NMS_GRADIENT) return TOED_ERR_UNSUPPORTED;
    if (prm->out_dtype != TOED_F32 && prm->out_dtype != TOED_F64) return TOED_ERR_INVALID_ARG;
    const int r = radius_of(prm);
    if (r < 1 || r > TOED_MAX_RADIUS) return TOED_ERR_UNSUPPORTED;
    long long tot = 0;
    for (int i = 0; i < n; ++i) {
        const toed_grad_image& g = items[i];
        if (!g.pixels || !g.grad_pixels || g.height <= 0 || g.width <= 0 || g.pitch < g.width || g.n_edgels < 0)
            return TOED_ERR_INVALID_ARG;
        if (g.n_edgels > 0 && (!g.grid_index || !g.grad_edgels)) return TOED_ERR_INVALID_ARG;
        if (g.dtype != TOED_U8 && g.dtype != TOED_F32) return TOED_ERR_UNSUPPORTED;
        tot += g.n_edgels;
    }
    if (tot >= (1LL << 31)) return TOED_ERR_UNSUPPORTED;
    int prev = 0;
    TOED_CU(cudaGetDevice(&prev));
    if (prev != c->device) TOED_CU(cudaSetDevice(c->device));
    toed_status st = TOED_OK;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        cudaError_t e = cudaMemsetAsync(grad_sigma, 0, sizeof(double), stream);
        for (int i0 = 0; i0 < n && e == cudaSuccess; i0 += kBatchMax)
            e = backward_launch(items + i0, std::min(kBatchMax, n - i0), prm, r, grad_sigma, stream);
        if (e != cudaSuccess) {
            g_last_cuda_error = std::string("backward: ") + cudaGetErrorString(e);
            st = TOED_ERR_CUDA;
        }
    }
    if (prev != c->device) cudaSetDevice(prev);
    return st;
}
