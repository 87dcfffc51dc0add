"""GB300-native Third-Order Edge Detector (TOED) hot path.

Python host mirror of the reference's detection interface over the C ABI in
include/toed_gb300.h.  The compute path is the CUDA library
``libtoed_gb300.so`` built in-tree for sm_103a by ``build.py``; there is no
CPU fallback: every entry point raises if the library is not built or no GPU
is present.  PyTorch is used only for device memory and streams.

Public API (names follow the reference):

* ``ThirdOrderEdgeDetectionGPU``  -- class mirror of the reference's
  ThirdOrderEdgeDetectionGPU<T> (gpu_toed.hpp:21-74): ctor(device, H, W,
  kernel_size, sigma), preprocessing(image), convolve_img(),
  non_maximum_suppresion() -> N, with ``TOED_edges`` / ``time_conv`` /
  ``time_nms``.
* ``detect`` / ``detect_batch``   -- functional form on torch tensors.
* ``Detector``                    -- reusable context (scratch, CUDA graphs).
"""
from __future__ import annotations

import ctypes
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# TOED_LIBRARY selects another build of the library (the bounds-checked
# libtoed_gb300_debug.so, in a process of its own); default: the release build
LIB_PATH = os.environ.get("TOED_LIBRARY") or os.path.join(HERE, "libtoed_gb300.so")
LIB_DEBUG_PATH = os.path.join(HERE, "libtoed_gb300_debug.so")

TOED_OK, TOED_ERR_INVALID_ARG, TOED_ERR_CAPACITY, TOED_ERR_CUDA, TOED_ERR_TIMEOUT, \
    TOED_ERR_UNSUPPORTED, TOED_ERR_CAPTURE = range(7)
TOED_U8, TOED_F32, TOED_F64 = 0, 1, 2
TOED_HYBRID, TOED_FP32 = 0, 1
TOED_ORI_GRID, TOED_ORI_QAD = 0, 1
TOED_NMS_GRADIENT, TOED_NMS_TO_NORMAL = 0, 1
TOED_FLAG_OVER_CAPACITY, TOED_FLAG_STAGING_FULL, TOED_FLAG_TIMEOUT, TOED_FLAG_BOUNDS = 1, 2, 4, 8
MAX_RADIUS = 12

# exported C symbols (checked by tests against include/toed_gb300.h)
C_SYMBOLS = [
    "toed_params_default", "toed_status_string", "toed_last_cuda_error", "toed_create",
    "toed_destroy", "toed_reserve", "toed_detect", "toed_detect_batch", "toed_device_flags",
    "toed_convolve_planes", "toed_convolve_planes_direct", "toed_nms_planes", "toed_profile_begin", "toed_profile_end",
    "toed_subpix_to_correct_batch", "toed_detect_noalloc", "toed_backward_batch", "toed_autotune",
    "toed_set_tuning", "toed_detect_host_batch", "toed_edgels_to_columns", "toed_write_edgels_txt",
]


class ToedError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({status})")


class toed_image(ctypes.Structure):
    _fields_ = [
        ("pixels", ctypes.c_void_p), ("height", ctypes.c_int), ("width", ctypes.c_int),
        ("pitch", ctypes.c_int), ("dtype", ctypes.c_int), ("edgels", ctypes.c_void_p),
        ("capacity", ctypes.c_int), ("count", ctypes.c_void_p), ("grid_index", ctypes.c_void_p),
    ]


class toed_params(ctypes.Structure):
    _fields_ = [
        ("sigma", ctypes.c_float), ("radius", ctypes.c_int), ("threshold", ctypes.c_float),
        ("border", ctypes.c_int), ("out_dtype", ctypes.c_int), ("precision", ctypes.c_int),
        ("orientation", ctypes.c_int), ("nms_direction", ctypes.c_int),
    ]


class toed_grad_image(ctypes.Structure):
    _fields_ = [
        ("pixels", ctypes.c_void_p), ("height", ctypes.c_int), ("width", ctypes.c_int),
        ("pitch", ctypes.c_int), ("dtype", ctypes.c_int), ("n_edgels", ctypes.c_int),
        ("grid_index", ctypes.c_void_p), ("grad_edgels", ctypes.c_void_p), ("grad_pixels", ctypes.c_void_p),
    ]


class toed_edgemap(ctypes.Structure):
    _fields_ = [
        ("E", ctypes.c_void_p), ("theta", ctypes.c_void_p), ("height", ctypes.c_int),
        ("width", ctypes.c_int), ("pitch", ctypes.c_int), ("dtype", ctypes.c_int),
        ("edgels", ctypes.c_void_p), ("capacity", ctypes.c_int), ("count", ctypes.c_void_p),
        ("TO_E", ctypes.c_void_p), ("TO_O", ctypes.c_void_p),
    ]


class toed_subpix_params(ctypes.Structure):
    _fields_ = [
        ("thresh", ctypes.c_float), ("sigma", ctypes.c_float), ("nbr_radius", ctypes.c_float),
        ("out_dtype", ctypes.c_int), ("precision", ctypes.c_int), ("interp_n", ctypes.c_int),
    ]


class toed_host_image(ctypes.Structure):
    _fields_ = [
        ("pixels", ctypes.c_void_p), ("height", ctypes.c_int), ("width", ctypes.c_int),
        ("pitch", ctypes.c_int), ("dtype", ctypes.c_int), ("edgels", ctypes.c_void_p),
        ("capacity", ctypes.c_int), ("count", ctypes.c_void_p), ("grid_index", ctypes.c_void_p),
    ]


_STAGING_NAMES = ["plain", "tma", "async"]  # toed_tuning.staging 0, 1, 2


class toed_tuning(ctypes.Structure):
    _fields_ = [("strip_rows", ctypes.c_int), ("staging", ctypes.c_int), ("ms", ctypes.c_float)]


_LIB = None


def build(verbose: bool = False, debug: bool = False) -> str:
    """Compile libtoed_gb300.so (nvcc, sm_103a) in-tree; with ``debug`` the
    bounds-checked libtoed_gb300_debug.so."""
    sys.path.insert(0, HERE)
    try:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_toed_build", os.path.join(HERE, "build.py"))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        return m.build(verbose=verbose, debug=debug)
    finally:
        sys.path.remove(HERE)


def lib():
    """The loaded CUDA library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library not built: {LIB_PATH} (call build())")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        L.toed_status_string.restype = ctypes.c_char_p
        L.toed_status_string.argtypes = [ip]
        L.toed_last_cuda_error.restype = ctypes.c_char_p
        L.toed_params_default.argtypes = [ctypes.POINTER(toed_params), ctypes.c_float]
        L.toed_create.argtypes = [ctypes.POINTER(vp), ip]
        L.toed_destroy.argtypes = [vp]
        L.toed_reserve.argtypes = [vp, i64, i64, ip]
        L.toed_detect.argtypes = [vp, ctypes.POINTER(toed_image), ctypes.POINTER(toed_params), vp]
        L.toed_detect_batch.argtypes = [vp, ctypes.POINTER(toed_image), ip,
                                        ctypes.POINTER(toed_params), vp]
        L.toed_device_flags.argtypes = [vp, vp, ctypes.POINTER(ip)]
        L.toed_convolve_planes.argtypes = [vp, ip, ip, ip, ip, ctypes.c_float, ip, vp, ip, vp, vp, vp,
                                           vp, vp]
        L.toed_convolve_planes_direct.argtypes = L.toed_convolve_planes.argtypes
        L.toed_nms_planes.argtypes = [ip, ip, ip, vp, vp, vp, ctypes.c_float, ip, vp, vp, vp]
        L.toed_profile_begin.argtypes = [vp]
        L.toed_profile_end.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ip)]
        L.toed_subpix_to_correct_batch.argtypes = [vp, ctypes.POINTER(toed_edgemap), ip,
                                                   ctypes.POINTER(toed_subpix_params), vp]
        L.toed_detect_noalloc.argtypes = [ctypes.POINTER(toed_image), ctypes.POINTER(toed_params), vp]
        L.toed_autotune.argtypes = [vp, ctypes.POINTER(toed_image), ip, ctypes.POINTER(toed_params), ip, vp,
                                    ctypes.POINTER(toed_tuning)]
        L.toed_set_tuning.argtypes = [vp, ctypes.POINTER(toed_params), ctypes.POINTER(toed_tuning)]
        L.toed_edgels_to_columns.argtypes = [vp, ip, ip, vp, vp]
        L.toed_write_edgels_txt.argtypes = [ctypes.c_char_p, vp, ip, ip, ip]
        L.toed_detect_host_batch.argtypes = [vp, ctypes.POINTER(toed_host_image), ip, ctypes.POINTER(toed_params),
                                             ip, vp]
        L.toed_backward_batch.argtypes = [vp, ctypes.POINTER(toed_grad_image), ip, ctypes.POINTER(toed_params),
                                          vp, vp]
        for name in C_SYMBOLS:
            if name not in ("toed_status_string", "toed_last_cuda_error", "toed_params_default"):
                getattr(L, name).restype = ip
        L.toed_params_default.restype = None
        _LIB = L
    return _LIB


def status_string(st: int) -> str:
    try:
        return lib().toed_status_string(int(st)).decode()
    except Exception:  # library not loadable: still give a readable message
        return {0: "ok", 1: "invalid argument", 2: "capacity exceeded", 3: "CUDA error",
                4: "device wait timed out", 5: "unsupported configuration",
                6: "scratch must grow during stream capture"}.get(int(st), "unknown")


def _check(st: int, what: str):
    if st != TOED_OK:
        msg = what
        if st == TOED_ERR_CUDA:
            msg += " [" + lib().toed_last_cuda_error().decode() + "]"
        raise ToedError(st, msg)


_PROBE = None


def peak_probe(kind: int = 0, iters: int = 200000, stream=None) -> float:
    """Measured FP32 (kind 0) or FP64 (kind 1) FMA rate in TFLOP/s, from the
    measurement library libtoed_probe.so (built by build(); not part of the
    detector's C ABI)."""
    global _PROBE
    t = _torch()
    if _PROBE is None:
        path = os.path.join(HERE, "libtoed_probe.so")
        if not os.path.exists(path):
            raise RuntimeError(f"probe library not built: {path} (call build())")
        _PROBE = ctypes.CDLL(path)
        _PROBE.toed_peak_probe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        _PROBE.toed_peak_probe.restype = ctypes.c_int
    s = stream if stream is not None else t.cuda.current_stream()
    out = ctypes.c_double(0.0)
    _check(_PROBE.toed_peak_probe(int(kind), int(iters), ctypes.c_void_p(s.cuda_stream), ctypes.byref(out)),
           "toed_peak_probe")
    return out.value


def default_radius(sigma: float) -> int:
    """r = ceil(4 sigma): kernel 17 at sigma 2 (cpu_toed.cpp:131, main_cpu_DP.cpp:182)."""
    return int(math.ceil(4.0 * sigma))


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("TOED GB300 path needs a CUDA device; there is no CPU fallback")
    return torch


def make_params(sigma=2.0, radius=0, threshold=2.0, border=10, out_dtype=TOED_F32,
                precision=TOED_HYBRID, orientation=TOED_ORI_GRID, nms_direction=TOED_NMS_GRADIENT) -> toed_params:
    """orientation: TOED_ORI_GRID (0, the C++ detector) or TOED_ORI_QAD (1,
    the MATLAB quick-and-dirty mode).  nms_direction: TOED_NMS_GRADIENT (0,
    the reference) or TOED_NMS_TO_NORMAL (1, NMS and peak fit along the
    corrected normal)."""
    return toed_params(float(sigma), int(radius), float(threshold), int(border), int(out_dtype),
                       int(precision), int(orientation), int(nms_direction))


class HostBatch:
    """A host-memory batch described once (Detector.host_batch): the C array
    of toed_host_image for toed_detect_host_batch plus references keeping the
    tensors alive."""

    def __init__(self, det, images, outs):
        t = det.torch
        self.det, self.images, self.outs = det, list(images), list(outs)
        if len(self.images) != len(self.outs):
            raise ValueError("one output set per image")
        arr = (toed_host_image * len(self.images))()
        for k, (im, o) in enumerate(zip(self.images, self.outs)):
            if im.dim() != 2 or im.device.type != "cpu" or im.stride(1) != 1:
                raise ValueError("host images must be 2-D CPU tensors with contiguous rows")
            dt = TOED_U8 if im.dtype == t.uint8 else (TOED_F32 if im.dtype == t.float32 else None)
            if dt is None:
                raise ValueError("image dtype must be uint8 or float32")
            H, W = im.shape
            arr[k] = toed_host_image(im.data_ptr(), H, W, im.stride(0), dt, o["edgels"].data_ptr(), o["capacity"],
                                     o["count"].data_ptr(),
                                     o["index"].data_ptr() if o.get("index") is not None else None)
        self.arr = arr

    def run(self, params: toed_params, chunks=None, stream=None):
        """chunks: copy groups (None: one image per group, the fastest for
        page-locked images; 1: page-locked images read in place)."""
        det = self.det
        if chunks is None:
            chunks = len(self.images)
        s = stream if stream is not None else det.torch.cuda.current_stream(det.device)
        _check(lib().toed_detect_host_batch(det._ctx, self.arr, len(self.images), ctypes.byref(params), int(chunks),
                                            ctypes.c_void_p(s.cuda_stream)), "toed_detect_host_batch")


class Detector:
    """A detection context on one device: owns the scratch of the fused
    kernel and (optionally) caches CUDA graphs of fixed batches."""

    def __init__(self, device: int = 0):
        self.torch = _torch()
        self.device = int(device)
        self._ctx = ctypes.c_void_p()
        with self.torch.cuda.device(self.device):
            _check(lib().toed_create(ctypes.byref(self._ctx), self.device), "toed_create")

    def close(self):
        if self._ctx:
            lib().toed_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, max_pixels: int, max_edgels: int, max_images: int):
        _check(lib().toed_reserve(self._ctx, int(max_pixels), int(max_edgels), int(max_images)),
               "toed_reserve")

    def profile_begin(self):
        """Time the fused detection kernel of every following call."""
        _check(lib().toed_profile_begin(self._ctx), "toed_profile_begin")

    def profile_end(self):
        """(total kernel ms, launches) since profile_begin()."""
        ms, n = ctypes.c_double(0.0), ctypes.c_int(0)
        _check(lib().toed_profile_end(self._ctx, ctypes.byref(ms), ctypes.byref(n)), "toed_profile_end")
        return ms.value, n.value

    def flags(self, stream=None) -> int:
        f = ctypes.c_int(0)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        _check(lib().toed_device_flags(self._ctx, ctypes.c_void_p(s.cuda_stream), ctypes.byref(f)),
               "toed_device_flags")
        return f.value

    # ------------------------------------------------------------------
    def alloc_outputs(self, shapes, capacity=None, out_dtype=TOED_F32, index=True):
        """Edgel / count / index buffers for images of the given (H, W)."""
        t = self.torch
        dt = t.float64 if out_dtype == TOED_F64 else t.float32
        outs = []
        for (H, W) in shapes:
            cap = int(capacity) if capacity is not None else 4 * H * W
            outs.append({
                "edgels": t.empty((max(cap, 1), 4), dtype=dt, device=f"cuda:{self.device}"),
                "count": t.zeros(1, dtype=t.int32, device=f"cuda:{self.device}"),
                "index": t.empty(max(cap, 1), dtype=t.int32, device=f"cuda:{self.device}")
                if index else None,
                "capacity": cap,
            })
        return outs

    def _image_struct(self, img, out):
        t = self.torch
        if img.dim() != 2 or img.device.type != "cuda":
            raise ValueError("images must be 2-D CUDA tensors")
        if img.dtype == t.uint8:
            dt = TOED_U8
        elif img.dtype == t.float32:
            dt = TOED_F32
        else:
            raise ValueError("image dtype must be uint8 or float32")
        if img.stride(1) != 1:
            raise ValueError("image rows must be contiguous")
        H, W = img.shape
        return toed_image(img.data_ptr(), H, W, img.stride(0), dt, out["edgels"].data_ptr(),
                          out["capacity"], out["count"].data_ptr(),
                          out["index"].data_ptr() if out.get("index") is not None else None)

    def detect_into(self, images, outs, params: toed_params, stream=None):
        """Launch detection of ``images`` into preallocated ``outs`` (async)."""
        n = len(images)
        arr = (toed_image * n)(*[self._image_struct(im, o) for im, o in zip(images, outs)])
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        _check(lib().toed_detect_batch(self._ctx, arr, n, ctypes.byref(params),
                                       ctypes.c_void_p(s.cuda_stream)), "toed_detect_batch")

    def autotune(self, images, outs, params: toed_params, reps: int = 3, stream=None) -> dict:
        """Time every candidate launch shape on this batch and keep the
        fastest for later calls with the same radius and precision
        (synchronous; the outputs hold the last run)."""
        n = len(images)
        arr = (toed_image * n)(*[self._image_struct(im, o) for im, o in zip(images, outs)])
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        best = toed_tuning()
        _check(lib().toed_autotune(self._ctx, arr, n, ctypes.byref(params), int(reps),
                                   ctypes.c_void_p(s.cuda_stream), ctypes.byref(best)), "toed_autotune")
        return {"strip_rows": best.strip_rows, "staging": _STAGING_NAMES[best.staging], "ms": best.ms}

    def set_tuning(self, params: toed_params, strip_rows=None, staging="tma"):
        """Install a launch shape (strip_rows None: the built-in heuristic);
        staging: "tma", "async" or "plain" (True / False mean "tma" / "plain")."""
        if isinstance(staging, bool):
            staging = "tma" if staging else "plain"
        t = toed_tuning(int(strip_rows), _STAGING_NAMES.index(staging), 0.0) if strip_rows is not None else None
        _check(lib().toed_set_tuning(self._ctx, ctypes.byref(params), ctypes.byref(t) if t is not None else None),
               "toed_set_tuning")

    def alloc_host_outputs(self, shapes, capacity=None, out_dtype=TOED_F32, index=False, pin=True):
        """Page-locked host edgel / count (/ index) buffers for detect_host."""
        t = self.torch
        dt = t.float64 if out_dtype == TOED_F64 else t.float32
        outs = []
        for (H, W) in shapes:
            cap = int(capacity) if capacity is not None else 4 * H * W
            o = {"edgels": t.empty((max(cap, 1), 4), dtype=dt), "count": t.zeros(1, dtype=t.int32),
                 "index": t.empty(max(cap, 1), dtype=t.int32) if index else None, "capacity": cap}
            if pin:
                o = {k: (v.pin_memory() if isinstance(v, t.Tensor) else v) for k, v in o.items()}
            outs.append(o)
        return outs

    def host_batch(self, images, outs):
        """Prepare a host-memory batch once for repeated detect_host calls on
        the same buffers (a serving loop's fixed page-locked staging): the
        returned object holds the images and outputs alive and the C array of
        toed_host_image describing them, so each call is one C call."""
        return HostBatch(self, images, outs)

    def detect_host(self, images, outs=None, params: toed_params = None, chunks=None, stream=None):
        """Detect edgels in images held in host memory (2-D CPU tensors,
        page-locked for full speed) into host buffers from
        alloc_host_outputs: copies in, detection and copies out are
        pipelined over ``chunks`` groups (synchronous; None: one image per
        group).  ``images`` may be a HostBatch from host_batch() (then
        ``outs`` is None)."""
        if params is None:
            raise ValueError("params required (make_params)")
        hb = images if isinstance(images, HostBatch) else HostBatch(self, images, outs)
        hb.run(params, chunks, stream)

    def capture(self, images, outs, params: toed_params, warmup: int = 1):
        """Capture detect_into(images, outs, params) in a CUDA graph (the
        persistent detection launch plus the ordering pass) and return it;
        ``graph.replay()`` re-runs the batch on the same buffers with no host
        work.  Scratch is reserved first, so nothing allocates under capture."""
        t = self.torch
        npx = sum(int(im.numel()) for im in images)
        self.reserve(npx, sum(int(o["capacity"]) for o in outs), len(images))
        s = t.cuda.Stream(self.device)
        s.wait_stream(t.cuda.current_stream(self.device))
        with t.cuda.stream(s):
            for _ in range(warmup):
                self.detect_into(images, outs, params, s)
        s.synchronize()
        g = t.cuda.CUDAGraph()
        with t.cuda.graph(g, stream=s):
            self.detect_into(images, outs, params, s)
        t.cuda.current_stream(self.device).wait_stream(s)
        return g

    def detect_batch(self, images, sigma=2.0, threshold=2.0, radius=0, border=10,
                     out_dtype=TOED_F32, precision=TOED_HYBRID, capacity=None, index=True,
                     stream=None, orientation=TOED_ORI_GRID, nms_direction=TOED_NMS_GRADIENT):
        """Detect edgels in a list of 2-D CUDA tensors.  Returns a list of
        dicts with ``edgels`` (N x 4: x, y, orientation, strength) and,
        with ``index``, the 2x-grid linear index of each edgel."""
        p = make_params(sigma, radius, threshold, border, out_dtype, precision, orientation, nms_direction)
        outs = self.alloc_outputs([tuple(im.shape) for im in images], capacity, out_dtype, index)
        self.detect_into(images, outs, p, stream)
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        s.synchronize()
        res = []
        for o in outs:
            n = int(o["count"].item())
            m = min(n, o["capacity"])
            r = {"count": n, "edgels": o["edgels"][:m]}
            if index:
                r["index"] = o["index"][:m]
            res.append(r)
        return res

    def detect(self, image, **kw):
        return self.detect_batch([image], **kw)[0]

    def backward_batch(self, images, indices, grad_edgels, sigma=2.0, radius=0, out_dtype=TOED_F32,
                       stream=None):
        """Adjoint of detect_batch with the selection frozen: given the
        forward's images, its per-image grid indices and dL/d(edgels)
        (N x 4 each), returns (dL/dimages as float32 tensors, dL/dsigma)."""
        t = self.torch
        dev = f"cuda:{self.device}"
        items, grads = [], []
        gdt = t.float64 if out_dtype == TOED_F64 else t.float32
        keep = []
        for im, idx, ge in zip(images, indices, grad_edgels):
            if im.stride(1) != 1:
                raise ValueError("image rows must be contiguous")
            H, W = im.shape
            gi = idx.to(device=dev, dtype=t.int32).contiguous()
            go = ge.to(device=dev, dtype=gdt).contiguous()
            gp = t.empty((H, W), dtype=t.float32, device=dev)
            keep += [gi, go]
            grads.append(gp)
            items.append(toed_grad_image(im.data_ptr(), H, W, im.stride(0),
                                         TOED_U8 if im.dtype == t.uint8 else TOED_F32, int(gi.numel()),
                                         gi.data_ptr() if gi.numel() else None,
                                         go.data_ptr() if go.numel() else None, gp.data_ptr()))
        arr = (toed_grad_image * len(items))(*items)
        gs = t.empty(1, dtype=t.float64, device=dev)  # cleared by toed_backward_batch
        p = make_params(sigma, radius, 2.0, 10, out_dtype)
        s = stream if stream is not None else t.cuda.current_stream(self.device)
        _check(lib().toed_backward_batch(self._ctx, arr, len(items), ctypes.byref(p), ctypes.c_void_p(gs.data_ptr()),
                                         ctypes.c_void_p(s.cuda_stream)), "toed_backward_batch")
        return grads, gs

    def subpix_to_correct_batch(self, maps, thresh=0.2, sigma=2.0, nbr_radius=2.0, thetas=None,
                                out_dtype=TOED_F32, precision=TOED_HYBRID, capacity=None, dense=True,
                                stream=None, interp_n=0):
        """Subpixel TO correction of dense edge maps (2-D CUDA float32 /
        float64 tensors), the reference's SubpixelTOCorrectionCPU<T>; with
        ``interp_n`` > 0 on its 2^n work grid.  Returns dicts with ``edgels``
        (N x 4: x, y, orientation, strength) and, with ``dense``, ``TO_E`` /
        ``TO_O`` (original size)."""
        t = self.torch
        dt = t.float64 if out_dtype == TOED_F64 else t.float32
        dev = f"cuda:{self.device}"
        arr, outs = [], []
        for k, E in enumerate(maps):
            if E.dim() != 2 or E.dtype not in (t.float32, t.float64) or E.stride(1) != 1:
                raise ValueError("edge maps must be 2-D row-contiguous float32/float64 CUDA tensors")
            th = None if thetas is None else thetas[k]
            if th is not None and (th.dtype != E.dtype or th.stride() != E.stride() or th.shape != E.shape):
                raise ValueError("orientation map must match the edge map's dtype, shape and strides")
            h, w = E.shape
            cap = int(capacity) if capacity is not None else ((h - 1) * (1 << interp_n) + 1) * ((w - 1) * (1 << interp_n) + 1)
            o = {"edgels": t.empty((max(cap, 1), 4), dtype=dt, device=dev),
                 "count": t.zeros(1, dtype=t.int32, device=dev), "capacity": cap}
            if dense:
                o["TO_E"] = t.empty((h, w), dtype=dt, device=dev)
                o["TO_O"] = t.empty((h, w), dtype=dt, device=dev)
            outs.append(o)
            arr.append(toed_edgemap(E.data_ptr(), th.data_ptr() if th is not None else None, h, w,
                                    E.stride(0), TOED_F64 if E.dtype == t.float64 else TOED_F32,
                                    o["edgels"].data_ptr(), cap, o["count"].data_ptr(),
                                    o["TO_E"].data_ptr() if dense else None,
                                    o["TO_O"].data_ptr() if dense else None))
        a = (toed_edgemap * len(arr))(*arr)
        prm = toed_subpix_params(float(thresh), float(sigma), float(nbr_radius), int(out_dtype), int(precision),
                                 int(interp_n))
        s = stream if stream is not None else t.cuda.current_stream(self.device)
        _check(lib().toed_subpix_to_correct_batch(self._ctx, a, len(arr), ctypes.byref(prm),
                                                  ctypes.c_void_p(s.cuda_stream)), "toed_subpix_to_correct_batch")
        s.synchronize()
        res = []
        for o in outs:
            n = int(o["count"].item())
            r = {"count": n, "edgels": o["edgels"][:min(n, o["capacity"])]}
            if dense:
                r["TO_E"], r["TO_O"] = o["TO_E"], o["TO_O"]
            res.append(r)
        return res


_DEFAULT = {}


def _default_detector(device: int = 0) -> Detector:
    d = _DEFAULT.get(device)
    if d is None:
        d = _DEFAULT[device] = Detector(device)
    return d


def detect(image, sigma=2.0, **kw):
    """Functional single-image detection on a CUDA tensor."""
    dev = image.device.index or 0
    return _default_detector(dev).detect(image, sigma=sigma, **kw)


def detect_batch(images, sigma=2.0, **kw):
    dev = images[0].device.index or 0
    return _default_detector(dev).detect_batch(images, sigma=sigma, **kw)


def edgels_to_columns(edgels, stream=None):
    """The n x 4 CUDA edgel list (float32 or float64) as the column-major
    double array curvelet formation reads (main_cpu_DP.cpp:225-236):
    returns a (4, n) float64 CUDA tensor whose row j is column j."""
    import torch
    if edgels.device.type != "cuda" or edgels.dim() != 2 or edgels.shape[1] != 4 or not edgels.is_contiguous():
        raise ValueError("edgels must be a contiguous n x 4 CUDA tensor")
    dt = TOED_F64 if edgels.dtype == torch.float64 else TOED_F32
    n = edgels.shape[0]
    out = torch.empty((4, n), dtype=torch.float64, device=edgels.device)
    s = stream if stream is not None else torch.cuda.current_stream(edgels.device)
    _check(lib().toed_edgels_to_columns(ctypes.c_void_p(edgels.data_ptr()), dt, n, ctypes.c_void_p(out.data_ptr()),
                                        ctypes.c_void_p(s.cuda_stream)), "toed_edgels_to_columns")
    return out


def write_edgels_txt(path: str, edgels, precision: int = 10):
    """Write a host n x 4 list (numpy float32/float64) in the reference's text
    format: precision 6 = data_final_output_cpu.txt (cpu_toed.cpp:556-580),
    10 = data_final_output_gpu.txt (gpu_toed.hpp:452-478)."""
    import numpy as np
    a = np.ascontiguousarray(edgels)
    if a.ndim != 2 or a.shape[1] != 4 or a.dtype not in (np.float32, np.float64):
        raise ValueError("edgels must be an n x 4 float32 or float64 array")
    dt = TOED_F64 if a.dtype == np.float64 else TOED_F32
    _check(lib().toed_write_edgels_txt(os.fsencode(path), a.ctypes.data_as(ctypes.c_void_p), dt, a.shape[0],
                                       int(precision)), "toed_write_edgels_txt")


class ThirdOrderEdgeDetectionGPU:
    """Mirror of the reference class ThirdOrderEdgeDetectionGPU<T>
    (gpu_toed.hpp:21-74; ctor gpu_toed.hpp:79-135).

    ``dtype`` plays the role of T: "float" gives float32 edgels, "double"
    float64 edgels (x, y keep FP64 positions).  ``sigma`` may be fractional
    (the reference stores an int, gpu_toed.hpp:30).  The file written by the
    reference's non_maximum_suppresion (data_final_output_gpu.txt,
    gpu_toed.hpp:439) is written only when ``output_dir`` is set.
    """

    num_of_edge_data = 4

    def __init__(self, device: int, H: int, W: int, kernel_size: int = 17, sigma: float = 2,
                 dtype: str = "float"):
        self.torch = _torch()
        self.device_id, self.img_height, self.img_width = int(device), int(H), int(W)
        self.kernel_sz = int(kernel_size)
        self.g_sig = sigma
        self.dtype = dtype
        self.edge_pt_list_idx = 0
        self.time_conv = 0.0
        self.time_nms = 0.0
        self.output_dir = None
        self.TOED_edges = None
        self._det = _default_detector(self.device_id)
        self._img = None
        self._res = None

    def set_output_dir(self, d: str):
        self.output_dir = d or "./output_files"

    def preprocessing(self, image):
        """image: HxW uint8/float array or tensor (the reference reads uint8,
        gpu_toed.hpp:141-231)."""
        t = self.torch
        if not isinstance(image, t.Tensor):
            image = t.as_tensor(image)
        if image.dtype not in (t.uint8, t.float32):
            image = image.to(t.float32)
        if tuple(image.shape) != (self.img_height, self.img_width):
            raise ValueError("image shape does not match the constructor's H, W")
        self._img = image.to(f"cuda:{self.device_id}").contiguous()

    def convolve_img(self):
        """Runs the fused detection (the reference's convolution + NMS
        kernels); ``time_conv`` gets its device time in ms."""
        t = self.torch
        if self._img is None:
            raise RuntimeError("preprocessing() must be called first")
        r = (self.kernel_sz - 1) // 2
        od = TOED_F64 if self.dtype == "double" else TOED_F32
        p = make_params(self.g_sig, r, 2.0, 10, od, TOED_HYBRID)
        outs = self._det.alloc_outputs([(self.img_height, self.img_width)], None, od, True)
        st, en = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        st.record()
        self._det.detect_into([self._img], outs, p)
        en.record()
        en.synchronize()
        self.time_conv = st.elapsed_time(en)
        self._res = outs[0]

    def non_maximum_suppresion(self, TOED_edges=None) -> int:
        """Returns N and fills ``TOED_edges`` (N x 4; also copied into the
        caller's array when one is passed, as gpu_toed.hpp:327-332)."""
        if self._res is None:
            raise RuntimeError("convolve_img() must be called first")
        t0 = self.torch.cuda.Event(enable_timing=True)
        t1 = self.torch.cuda.Event(enable_timing=True)
        t0.record()
        n = int(self._res["count"].item())
        m = min(n, self._res["capacity"])
        edges = self._res["edgels"][:m].cpu().numpy()
        t1.record()
        t1.synchronize()
        self.time_nms = t0.elapsed_time(t1)
        self.edge_pt_list_idx = n
        self.TOED_edges = edges
        if TOED_edges is not None:
            TOED_edges[:m] = edges
        if self.output_dir:
            os.makedirs(self.output_dir, exist_ok=True)
            with open(os.path.join(self.output_dir, "data_final_output_gpu.txt"), "w") as f:
                for row in edges:
                    f.write("".join(f"{v:.10g}\t" for v in row) + "\n")
        return n


def differentiable_detect(images, sigma, threshold=2.0, radius=0, detector=None):
    """Edgels of a batch as a differentiable function of the pixels and sigma.

    ``images``: (B, H, W) float32 CUDA tensor; ``sigma``: 0-d tensor (may
    require grad).  Returns (edgels (N, 4) [x, y, orientation, strength],
    counts (B,), grid_index (N,)) with the edgels of all images
    concatenated.  The backward is the hand-written adjoint
    (toed_backward_batch) with the selection held fixed."""
    import torch

    det = detector or _default_detector(images.device.index or 0)

    class _Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, imgs, sig):
            s = float(sig.detach().cpu())
            res = det.detect_batch(list(imgs), sigma=s, threshold=threshold, radius=radius, index=True)
            counts = torch.tensor([r["count"] for r in res], dtype=torch.int64)
            edg = torch.cat([r["edgels"] for r in res])
            idx = torch.cat([r["index"] for r in res])
            ctx.save_for_backward(imgs)
            ctx.sigma = s
            ctx.sig_meta = (sig.dtype, sig.device)
            ctx.idx = [r["index"] for r in res]
            ctx.counts = counts.tolist()
            ctx.mark_non_differentiable(idx, counts)
            return edg, idx, counts

        @staticmethod
        def backward(ctx, g_edg, g_idx, g_cnt):
            (imgs,) = ctx.saved_tensors
            splits = torch.split(g_edg.contiguous(), ctx.counts)
            grads, gs = det.backward_batch(list(imgs), ctx.idx, list(splits), sigma=ctx.sigma, radius=radius)
            gi = torch.stack(grads) if ctx.needs_input_grad[0] else None
            gsig = gs.reshape(()).to(dtype=ctx.sig_meta[0], device=ctx.sig_meta[1]) if ctx.needs_input_grad[1] else None
            return gi, gsig

    sig = sigma if isinstance(sigma, torch.Tensor) else torch.tensor(float(sigma))
    edg, idx, counts = _Fn.apply(images, sig)
    return edg, counts, idx
