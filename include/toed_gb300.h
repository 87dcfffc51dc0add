/*
 * toed_gb300.h -- C ABI of the GB300-native Third-Order Edge Detector (TOED).
 *
 * Plain C: pointers, sizes and a cudaStream_t; no C++ or framework types.
 * Every entry point returns a toed_status immediately (host-side argument
 * and launch errors).  Device-side conditions (an image with more edgels
 * than its capacity, a staging overflow) are recorded in device flags that
 * toed_device_flags() reads back.
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   toed_detect / toed_detect_batch
 *       ThirdOrderEdgeDetectionGPU<T>::convolve_img()            gpu_toed.hpp:340-413
 *       ThirdOrderEdgeDetectionGPU<T>::non_maximum_suppresion()  gpu_toed.hpp:415-441
 *       (with the host compaction build_edge_list               gpu_toed.hpp:313-338)
 *       and its CPU twin ThirdOrderEdgeDetectionCPU<T>          cpu_toed.cpp:128-545
 *       Output: N x 4 edgels [x, y, orientation, strength], row-major over
 *       the 2x grid, x = (pos_x - 1)/2, y = (pos_y - 1)/2 (cpu_toed.cpp:510-538).
 *   toed_convolve_planes
 *       gpu_convolve(device_id, h, w, interp_h, interp_w, dev_img, dev_Ix, ...)
 *                                                               gpu_kernels.hpp:24-45
 *   toed_convolve_planes_direct
 *       the same call, the reference kernel's summation structure
 *                                               gpu_convolve.cu:8-349
 *   toed_nms_planes
 *       gpu_nms(device_id, interp_h, interp_w, dev_Ix, dev_Iy, dev_I_grad_mag,
 *               dev_subpix_pos_x_map, dev_subpix_pos_y_map)     gpu_kernels.hpp:48-63
 *   toed_subpix_to_correct_batch
 *       SubpixelTOCorrectionCPU<T>::estimate_orientation() / run()
 *                                     subpix_TO_correction/subpix_to_correction.hpp:80-96
 *   toed_backward
 *       no reference counterpart (the reference has no gradients); adjoint of
 *       toed_detect with the selection mask held fixed.
 */
#ifndef TOED_GB300_H
#define TOED_GB300_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TOED_ABI_VERSION 2 /* 2: toed_params.nms_direction */
#define TOED_MAX_RADIUS 12 /* kernel half-width r = ceil(4 sigma) <= 12, i.e. sigma <= 3 */

typedef enum toed_status {
    TOED_OK = 0,
    TOED_ERR_INVALID_ARG = 1, /* null pointer, bad size, sigma <= 0, r out of range ... */
    TOED_ERR_CAPACITY = 2,    /* scratch or output capacity too small (counts stay exact) */
    TOED_ERR_CUDA = 3,        /* a CUDA runtime call failed; see toed_last_cuda_error */
    TOED_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
    TOED_ERR_UNSUPPORTED = 5, /* e.g. radius above TOED_MAX_RADIUS, dtype not handled */
    TOED_ERR_CAPTURE = 6      /* scratch would have to grow while the stream is being captured */
} toed_status;

typedef enum toed_dtype {
    TOED_U8 = 0,  /* unsigned 8-bit pixels (the reference's input, cpu_toed.cpp:68,103) */
    TOED_F32 = 1, /* float32 pixels */
    TOED_F64 = 2  /* float64 (edgel output and compatibility planes only) */
} toed_dtype;

typedef enum toed_precision {
    TOED_HYBRID = 0, /* FP32 convolutions; per-edgel peak fit whose cancelling sums are formed from
                        exact differences of the FP32 magnitudes; edgels whose TO vector nearly
                        cancels get their derivatives and orientation recomputed in FP64 */
    TOED_FP32 = 1    /* everything FP32 (precision-study mode) */
} toed_precision;

/* Where the emitted third-order orientation is evaluated. */
typedef enum toed_orientation {
    TOED_ORI_GRID = 0, /* at the edgel's 2x-grid point (the C++ detector, cpu_toed.cpp:227-232) */
    TOED_ORI_QAD = 1   /* MATLAB "quick and dirty" mode (third_order_edge_detector.m:91-141): the nine
                          derivatives cubic-interpolated (interp2 'cubic', Keys a = -1/2) at the
                          subpixel point; positions and strengths unchanged */
} toed_orientation;

/* Direction of the subpixel NMS and its parabola peak fit. */
typedef enum toed_nms_direction {
    TOED_NMS_GRADIENT = 0, /* along the first-order gradient (Ix, Iy): the reference
                              (cpu_toed.cpp:411-489) */
    TOED_NMS_TO_NORMAL = 1 /* along the corrected normal, the unit third-order vector
                              (TO_Ix, TO_Iy) of cpu_toed.cpp:227-230 whose tangent is the
                              emitted orientation; same candidates (threshold, gradient
                              epsilon), same emitted orientation.  No reference counterpart;
                              grid orientation only, no adjoint */
} toed_nms_direction;

/* Device flags (toed_device_flags) */
#define TOED_FLAG_OVER_CAPACITY 0x1 /* some image found more edgels than its capacity */
#define TOED_FLAG_STAGING_FULL 0x2  /* the context staging buffer overflowed */
#define TOED_FLAG_TIMEOUT 0x4       /* a bounded wait for an input copy gave up (results incomplete) */
#define TOED_FLAG_BOUNDS 0x8        /* bounds-checked debug library only: an index check failed and the
                                       access was skipped */

typedef struct toed_ctx toed_ctx;

/* One image of a detection batch.  All pointers are device pointers. */
typedef struct toed_image {
    const void* pixels; /* height x pitch elements of `dtype`, row-major */
    int height;
    int width;
    int pitch;          /* elements between row starts, >= width */
    int dtype;          /* TOED_U8 or TOED_F32 */
    void* edgels;       /* capacity x 4 of params->out_dtype: x, y, orientation, strength */
    int capacity;       /* edgels the buffer holds; the reference sizes it (2H)(2W) */
    int* count;         /* 1 int: number of edgels found (exact even when > capacity) */
    int* grid_index;    /* optional (NULL): per edgel, 2x-grid linear index row*(2W)+col */
} toed_image;

typedef struct toed_params {
    float sigma;       /* Gaussian scale (reference: int 2, main_cpu_DP.cpp:183) */
    int radius;        /* half-width r; 0 -> ceil(4 sigma) (kernel 17 at sigma 2) */
    float threshold;   /* |grad I| <= threshold is skipped; reference literal 2 (cpu_toed.cpp:403) */
    int border;        /* NMS skips a border of this many 2x-grid points; reference 10 (cpu_toed.cpp:400) */
    int out_dtype;     /* TOED_F32 (16-byte edgels) or TOED_F64 (32-byte edgels) */
    int precision;     /* toed_precision */
    int orientation;   /* toed_orientation (TOED_ORI_GRID: the reference C++ detector) */
    int nms_direction; /* toed_nms_direction (TOED_NMS_GRADIENT: the reference) */
} toed_params;

/* Fill `p` with the reference's configuration for a given sigma. */
void toed_params_default(toed_params* p, float sigma);

const char* toed_status_string(toed_status s);
const char* toed_last_cuda_error(void); /* text of the last CUDA error seen by this thread */

/* Context: per-device scratch (work queue, staging, row-segment table).
 * Replaces the buffers ThirdOrderEdgeDetectionGPU allocates in its
 * constructor (gpu_toed.hpp:79-135); callers own images and outputs. */
toed_status toed_create(toed_ctx** ctx, int device);
toed_status toed_destroy(toed_ctx* ctx);
/* Pre-size scratch so that later calls (e.g. under stream capture) never
 * allocate: total pixels, total edgel capacity and images per call. */
toed_status toed_reserve(toed_ctx* ctx, long long max_pixels, long long max_edgels, int max_images);

/* Fused detection of one image / a batch of images of any sizes in one
 * persistent launch (plus a short ordering pass).  Asynchronous on
 * `stream`; graph-capturable once scratch is reserved. */
toed_status toed_detect(toed_ctx* ctx, const toed_image* image, const toed_params* params,
                        cudaStream_t stream);
toed_status toed_detect_batch(toed_ctx* ctx, const toed_image* images, int n_images,
                              const toed_params* params, cudaStream_t stream);

/* Synchronises `stream` and returns the OR of the device flags of the last
 * detection on this context (0 = all images fit their capacities). */
toed_status toed_device_flags(toed_ctx* ctx, cudaStream_t stream, int* flags);

/* Adjoint of toed_detect with the selection frozen (no reference counterpart:
 * the reference has no gradients).  For every edgel the forward emitted
 * (identified by the grid_index it wrote), given dL/d[x, y, orientation,
 * strength], writes dL/dpixel for the whole image and dL/dsigma of the whole batch
 * (*grad_sigma, a device double, is overwritten).
 * The NMS decisions (which 2x-grid points are edgels, and each one's sector)
 * are those of the forward and are not differentiated. */
typedef struct toed_grad_image {
    const void* pixels;       /* the forward's input (device) */
    int height, width, pitch, dtype;
    int n_edgels;             /* edgels of the forward (its count, at most its capacity) */
    const int* grid_index;    /* the forward's grid_index output (device), ascending */
    const void* grad_edgels;  /* n_edgels x 4 cotangents (device), params->out_dtype */
    float* grad_pixels;       /* height x width float32 (device, row pitch = width): overwritten */
} toed_grad_image;

/* params->orientation must be TOED_ORI_GRID (TOED_ERR_UNSUPPORTED otherwise). */
toed_status toed_backward_batch(toed_ctx* ctx, const toed_grad_image* items, int n_images,
                                const toed_params* params, double* grad_sigma, cudaStream_t stream);

/* Subpixel third-order correction of dense edge maps (the reference's
 * SubpixelTOCorrectionCPU<T>, subpix_TO_correction/subpix_to_correction.cpp,
 * at interp_n = 0).  All pointers are device pointers. */
typedef struct toed_edgemap {
    const void* E;      /* height x pitch edge map (probabilities), TOED_F32 or TOED_F64 */
    const void* theta;  /* optional orientation map in radians (same dtype/pitch); NULL ->
                           estimated from E (estimate_orientation, :307-375) */
    int height;         /* >= 2 */
    int width;          /* >= 2 */
    int pitch;          /* elements between row starts */
    int dtype;
    void* edgels;       /* capacity x 4 of out_dtype: x, y, orientation, strength (0-based px) */
    int capacity;
    int* count;         /* edgels after removing isolated ones (exact even past capacity) */
    void* TO_E;         /* optional dense height x width (out_dtype): strength at round(x, y) */
    void* TO_O;         /* optional dense height x width (out_dtype): orientation at round(x, y) */
} toed_edgemap;

typedef struct toed_subpix_params {
    float thresh;      /* NMS threshold on E (reference default 0.2; main_subpix_to_correction.cpp:147) */
    float sigma;       /* Gaussian scale; radius ceil(4 sigma) <= TOED_MAX_RADIUS */
    float nbr_radius;  /* drop edgels with no other edgel within this distance; <= 0 keeps all (default 2) */
    int out_dtype;     /* TOED_F32 or TOED_F64 */
    int precision;     /* TOED_HYBRID: orientation estimate in double-float arithmetic where NMS
                          candidates lie, peak fit on exact FP32 differences, correction vector as
                          a compensated FP32 dot product, FP64 near-tie max tests; TOED_FP32: FP32 */
    int interp_n;      /* 0..4: work on the 2^n grid ((h-1) 2^n + 1 rows), the map (and theta)
                          bilinearly resized onto it; positions in original pixels
                          (the reference's interp_n, subpix_to_correction.cpp:95-105, :224-244) */
} toed_subpix_params;

toed_status toed_subpix_to_correct_batch(toed_ctx* ctx, const toed_edgemap* maps, int n_maps,
                                         const toed_subpix_params* params, cudaStream_t stream);

/* Allocation-free detection (no counterpart in the reference).
 * For callers that cannot call cudaMalloc where they detect edges -- code
 * whose device memory is owned by a pool or arena, real-time loops that
 * forbid allocation after start-up, plug-in hosts that hand out only
 * pre-sized buffers -- and therefore cannot use a toed_ctx, whose scratch
 * grows on demand.  One image per call on the current device; the caller
 * passes the image and the output buffers as for toed_detect, and the same
 * image checks apply.  The scratch is a fixed array compiled into the
 * library (about 11 MB).  The CUDA runtime loads it lazily: the first call
 * on a device reserves it there (until the process exits) and looks up its
 * device address, so make that first call at start-up, before a pool or
 * arena claims the device's memory (else TOED_ERR_CUDA) and before any
 * stream capture.  Images above TOED_NOALLOC_MAX_DIM rows or columns or
 * TOED_NOALLOC_MAX_PIXELS pixels, or a capacity above
 * TOED_NOALLOC_MAX_EDGELS, return TOED_ERR_CAPACITY.  All calls share the
 * array: calls that overlap on the GPU (other streams or host threads on the
 * same device) race and must be serialised by the caller.  If the image has
 * more edgels than `capacity`, count is exact but the contents of edgels
 * and grid_index are undefined (entries may be missing or hold an earlier
 * call's data): size the capacity for the image, (2H)(2W) at most. */
#define TOED_NOALLOC_MAX_DIM 4096
#define TOED_NOALLOC_MAX_PIXELS (2048LL * 2048LL)
#define TOED_NOALLOC_MAX_EDGELS 262144
toed_status toed_detect_noalloc(const toed_image* image, const toed_params* params, cudaStream_t stream);

/* Detection of images held in host memory -- the reference's flow (copy the
 * image in, detect, copy the edgel list back, gpu_toed.hpp:141-231 and
 * :415-441) for a whole batch, pipelined: the batch is cut into `chunks`
 * groups of consecutive images, growing in pixel count, and the copy of
 * group k+1 to the device overlaps the detection of group k.  Page-locked
 * images, at most 64: one detection launch for the whole batch whose CTAs
 * wait (bounded) for their group's copy, which the call enqueues right after
 * the launch -- another host thread that waits for the whole device in that
 * moment (cudaDeviceSynchronize, cudaFree) can hold those copies back until
 * the wait gives up (TOED_ERR_TIMEOUT), so serialise such calls; with
 * CUDA_LAUNCH_BLOCKING or under a profiler this flow is not used.  With
 * chunks == 1 no copy at all (the kernel reads them in place through their
 * device mapping).  Pageable
 * images, or more than 64: one launch per group (streams of the context,
 * ordered by events).  Page-locked
 * output buffers (edgels, count,
 * grid_index) are written by the detection's ordering pass directly through
 * their device mapping; pageable ones are filled by copies per group once its
 * counts are read back.  Synchronous: returns when every count and list is in
 * host memory.  Device staging is kept in the context and grows on demand.
 * Page-locked image buffers give full copy speed.  Returns
 * TOED_ERR_TIMEOUT if a bounded device wait gave up; more edgels than
 * `capacity` show as count > capacity (the list holds the first capacity). */
typedef struct toed_host_image {
    const void* pixels; /* host: height x pitch elements of `dtype` */
    int height;
    int width;
    int pitch;          /* elements between row starts, >= width */
    int dtype;          /* TOED_U8 or TOED_F32 */
    void* edgels;       /* host: capacity x 4 of params->out_dtype */
    int capacity;
    int* count;         /* host: 1 int */
    int* grid_index;    /* optional host: capacity ints */
} toed_host_image;

toed_status toed_detect_host_batch(toed_ctx* ctx, const toed_host_image* images, int n_images,
                                   const toed_params* params, int chunks, cudaStream_t stream);

/* After detection (the reference's drivers; no kernel counterpart there).
 * toed_edgels_to_columns: the n x 4 device list (TOED_F32 or TOED_F64) as the
 * column-major n x 4 double array curvelet formation reads
 * (form_curvelet_process, main_cpu_DP.cpp:225-236), on the device.
 * toed_write_edgels_txt: a host list as the text file non_maximum_suppresion
 * writes -- each value followed by a tab, a newline per edgel, `precision`
 * significant digits: 6 for data_final_output_cpu.txt (cpu_toed.cpp:556-580),
 * 10 for data_final_output_gpu.txt (gpu_toed.hpp:452-478). */
toed_status toed_edgels_to_columns(const void* edgels, int dtype, int n, double* columns, cudaStream_t stream);
toed_status toed_write_edgels_txt(const char* path, const void* edgels, int dtype, int n, int precision);

/* Launch-shape autotuning (no counterpart in the reference, whose GPU path
 * has one fixed launch shape).  toed_autotune times each candidate -- strip
 * height 14, 30, 62, 126, 254, 510 or 1022 rows, input rows staged by TMA, by
 * per-thread async copies or by plain loads -- on the caller's batch with CUDA
 * events, `reps` timed runs
 * after one untimed run each, keeps the fastest in the context for this
 * radius, precision and launch size class -- floor(log2(pixels)) of each
 * launch of the batch (64 images at most per launch) -- and returns it; later
 * launches of the same class use it, launches of other classes keep the
 * built-in heuristic.
 * It is synchronous, runs the detection 21 * (reps + 1) times (the outputs hold
 * the last run; every candidate gives the same result bit for bit) and is
 * refused under stream capture.  toed_set_tuning installs a shape for every
 * size class (NULL restores the built-in heuristic). */
typedef struct toed_tuning {
    int strip_rows;  /* 16k - 2 for k in 1, 2, 4, ..., 64 */
    int staging;     /* input row staging: 1 TMA (when the image allows it), 2 per-thread async
                        copies two steps ahead (float32 images), 0 plain loads */
    float ms;        /* measured time of one detection of the batch (autotune output) */
} toed_tuning;

toed_status toed_autotune(toed_ctx* ctx, const toed_image* images, int n_images, const toed_params* params,
                          int reps, cudaStream_t stream, toed_tuning* best);
toed_status toed_set_tuning(toed_ctx* ctx, const toed_params* params, const toed_tuning* tuning);

/* Measurement hooks (used by bench.py).
 * toed_profile_begin: from now on every detection on `ctx` records a pair of
 * CUDA events just before and just after its fused detection kernel, on the
 * call's stream.  toed_profile_end: waits for the last pair, returns the sum
 * of the kernel times (ms) and the number of kernel launches, and stops. */
toed_status toed_profile_begin(toed_ctx* ctx);
toed_status toed_profile_end(toed_ctx* ctx, double* kernel_ms, int* launches);

/* Compatibility: the reference's dense two-kernel form.
 * toed_convolve_planes writes Ix, Iy, |grad I| and the TO orientation on the
 * 2x grid ((2h) x (2w) row-major, dtype planes_dtype = TOED_F32 or TOED_F64,
 * the latter computed in FP64 throughout); toed_nms_planes writes the subpixel
 * position maps (zero where no edgel), as gpu_convolve / gpu_nms do.
 * `taps` (optional, host) overrides the generated filters: 8 rows of 2r+3
 * doubles, G, Gx, Gxx, Gxxx then the +0.5-shifted set, entry k at offset
 * k-(r+1) -- the arrays the reference passes to gpu_convolve. */
toed_status toed_convolve_planes(const void* pixels, int dtype, int h, int w, int pitch,
                                 float sigma, int radius, const double* taps, int planes_dtype,
                                 void* Ix, void* Iy, void* grad_mag, void* orient,
                                 cudaStream_t stream);
/* The same planes, same arguments, summed the way the reference's
 * gpu_convolve_kernel sums them (gpu_convolve.cu:96-300): each of the nine
 * derivatives of each sub-grid as a full 2-D window -- (2r+1)^2 taps on
 * sub-grid (0,0), (2r+3)^2 elsewhere -- row offset outer, column offset
 * inner.  For callers that want the reference's summation order (its FP32
 * rounding pattern) and as the reference's single-image GPU form in
 * benchmarks; toed_convolve_planes gives the same planes separably at a
 * fraction of the cost. */
toed_status toed_convolve_planes_direct(const void* pixels, int dtype, int h, int w, int pitch,
                                        float sigma, int radius, const double* taps, int planes_dtype,
                                        void* Ix, void* Iy, void* grad_mag, void* orient,
                                        cudaStream_t stream);
toed_status toed_nms_planes(int planes_dtype, int interp_h, int interp_w, const void* Ix,
                            const void* Iy, const void* grad_mag, float threshold, int border,
                            void* pos_x_map, void* pos_y_map, cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* TOED_GB300_H */
