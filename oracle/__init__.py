"""CPU oracle for the TOED hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this package, and only as the checker (or, for the CPU baseline, as the timed
restatement of the reference's OpenMP path).  The CUDA library never imports
it; its product path fails loudly when the CUDA extension is missing.

Two native libraries sit behind it:

* ``oracle/liboracle.so`` -- the C restatement ``oracle/toed_oracle.c`` of the
  reference's FP64 CPU path (cpu_toed.cpp:128-545 and
  subpix_TO_correction/subpix_to_correction.cpp:195-736).  Built from
  committed source on any host (x86 here, aarch64 on the GPU host).
* ``oracle/_ref/libref_toed.so`` -- the reference's own cpu_toed.cpp and
  subpix_to_correction.cpp compiled where they lie (``make -C oracle ref``),
  only where the reference sources exist.  Used to pin the restatement and to
  generate the committed golden fixtures under tests/golden/.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_dp = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


REF_COPY = os.path.abspath(os.path.join(_HERE, "..", "baseline", "_ref", "src"))


def _has_sources(d) -> bool:
    return bool(d) and os.path.exists(os.path.join(d, "cpu_toed.cpp")) and \
        os.path.exists(os.path.join(d, "gpu_convolve.cu"))


def checkout_dir() -> str:
    """The reference checkout: the TOED_REF_DIR environment variable, else
    the recipe's default (may not exist on this host)."""
    env = os.environ.get("TOED_REF_DIR")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", _HERE, "refdir"], capture_output=True, text=True)
    return r.stdout.strip()


def ref_dir() -> str:
    """Where the reference builds read the reference's sources: the checkout
    where it exists, else the git-ignored copy baseline/_ref/src that
    ``make -C oracle refsrc`` made from it (it travels with the working tree
    to hosts that have no checkout)."""
    d = checkout_dir()
    return d if _has_sources(d) else REF_COPY


def ref_sources_present() -> bool:
    """True where the reference's sources can be compiled: its checkout, or
    the copy of its files in baseline/_ref/src."""
    return _has_sources(ref_dir())


def build(ref: bool = False, refgpu: bool = False) -> None:
    """Compile liboracle.so; with ``ref`` the reference's own CPU classes,
    with ``refgpu`` its GPU class and kernels (oracle/_ref).  Where the
    checkout exists, its files are first copied to baseline/_ref/src."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    if not (ref or refgpu):
        return
    d = ref_dir()
    if d != REF_COPY:
        subprocess.run(["make", "-s", "-C", _HERE, "refsrc", f"REF_DIR={d}"], check=True)
    targets = (["ref"] if ref else []) + (["refgpu"] if refgpu else [])
    subprocess.run(["make", "-s", "-j4", "-C", _HERE] + targets + [f"REF_DIR={d}"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.toed_oracle_taps.argtypes = [ctypes.c_double, ctypes.c_int, _dp]
        L.toed_oracle_detect.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, ctypes.c_double,
            ctypes.c_int, _dp, ctypes.c_long, _dp, _dp, _i64p]
        L.toed_oracle_detect.restype = ctypes.c_long
        L.toed_oracle_detect_ex.argtypes = L.toed_oracle_detect.argtypes + [ctypes.c_int]
        L.toed_oracle_detect_ex.restype = ctypes.c_long
        L.toed_oracle_detect_qad.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, ctypes.c_double,
            ctypes.c_int, _dp, ctypes.c_long, _i64p]
        L.toed_oracle_detect_qad.restype = ctypes.c_long
        L.toed_oracle_planes.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
        L.subpix_oracle_run.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp,
            ctypes.c_int, _dp, ctypes.c_long, _dp, _dp, _dp, _dp, _dp]
        L.subpix_oracle_run.restype = ctypes.c_long
        L.subpix_oracle_run_n.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
            _dp, ctypes.c_int, _dp, ctypes.c_long, _dp, _dp, _dp, _dp, _dp]
        L.subpix_oracle_run_n.restype = ctypes.c_long
        L.subpix_oracle_kernels.argtypes = [ctypes.c_double, _dp]
        L.subpix_oracle_kernels.restype = ctypes.c_int
        _LIB = L
    return _LIB


def default_radius(sigma: float) -> int:
    """Half-width r = ceil(4 sigma) (17 taps at sigma 2, cpu_toed.cpp:131)."""
    return int(math.ceil(4.0 * sigma))


def taps(sigma: float, r: int | None = None) -> np.ndarray:
    """(8, 2r+3) tap block: G, Gx, Gxx, Gxxx, then the +0.5-shifted set."""
    r = default_radius(sigma) if r is None else r
    out = np.zeros((8, 2 * r + 3), np.float64)
    lib().toed_oracle_taps(float(sigma), int(r), _ptr(out))
    return out


def detect(img, sigma: float = 2.0, r: int | None = None, tap_block=None, threshold: float = 2.0,
           nthreads: int = 0, planes: bool = False, orientation: str = "grid", nms: str = "gradient"):
    """FP64 TOED.  Returns dict(edges=(N,4), index=(N,) 2x-grid linear index
    [, planes=(4,2H,2W) Ix/Iy/mag/ori, posmaps=(3,2H,2W)]).
    orientation="qad": the MATLAB quick-and-dirty mode
    (third_order_edge_detector.m:91-141), derivatives cubic-interpolated at
    the subpixel point (no plane outputs).
    nms="to_normal": NMS and peak fit along the corrected normal (the
    third-order vector) instead of the gradient (cpu_toed.cpp:411-489), an
    extension beyond the reference."""
    if orientation not in ("grid", "qad"):
        raise ValueError(orientation)
    if nms not in ("gradient", "to_normal"):
        raise ValueError(nms)
    if nms == "to_normal" and orientation != "grid":
        raise ValueError("nms='to_normal' is defined with the grid orientation")
    img = np.ascontiguousarray(img, dtype=np.float64)
    H, W = img.shape
    r = default_radius(sigma) if r is None else r
    tb = None
    if tap_block is not None:
        tb = np.ascontiguousarray(tap_block, dtype=np.float64)
        assert tb.shape == (8, 2 * r + 3)
    cap = 4 * H * W
    edges = np.zeros((cap, 4), np.float64)
    index = np.zeros(cap, np.int64)
    if orientation == "qad":
        if planes:
            raise ValueError("orientation='qad' has no plane outputs")
        n = lib().toed_oracle_detect_qad(_ptr(img), H, W, float(sigma), int(r), _ptr(tb), float(threshold),
                                         int(nthreads), _ptr(edges), cap, index.ctypes.data_as(_i64p))
        return {"edges": edges[:n].copy(), "index": index[:n].copy()}
    pl = np.zeros((4, 2 * H, 2 * W), np.float64) if planes else None
    pm = np.zeros((3, 2 * H, 2 * W), np.float64) if planes else None
    n = lib().toed_oracle_detect_ex(_ptr(img), H, W, float(sigma), int(r), _ptr(tb), float(threshold),
                                    int(nthreads), _ptr(edges), cap, _ptr(pl), _ptr(pm),
                                    index.ctypes.data_as(_i64p), 1 if nms == "to_normal" else 0)
    out = {"edges": edges[:n].copy(), "index": index[:n].copy()}
    if planes:
        out["planes"] = pl
        out["posmaps"] = pm
    return out


def planes9(img, sigma: float = 2.0, r: int | None = None, nthreads: int = 0):
    """All nine derivative planes on the 2x grid: (9, 2H, 2W) in the order
    fx, fy, fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy."""
    img = np.ascontiguousarray(img, dtype=np.float64)
    H, W = img.shape
    r = default_radius(sigma) if r is None else r
    tb = taps(sigma, r)
    d9 = np.zeros((9, 2 * H, 2 * W), np.float64)
    lib().toed_oracle_planes(_ptr(img), H, W, int(r), _ptr(tb), int(nthreads), None, None, None,
                             None, _ptr(d9))
    return d9


def subpix_to_correct(E, thresh: float = 0.1, sigma: float = 2.0, nbr_radius: float = 2.0,
                      theta=None, nthreads: int = 0, dense: bool = False, debug: bool = False,
                      interp_n: int = 0):
    """FP64 subpixel TO correction on the 2^interp_n work grid.  Returns
    dict(edges=(N,4) [, TO_E, TO_O (original size)] [, nms=(4,hw,ww),
    theta=(hw,ww), planes10=(10,hw,ww) on the work grid])."""
    E = np.ascontiguousarray(E, dtype=np.float64)
    h, w = E.shape
    sc = 1 << max(int(interp_n), 0)
    hw, ww = (h - 1) * sc + 1, (w - 1) * sc + 1
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    cap = hw * ww
    edges = np.zeros((cap, 4), np.float64)
    TE = np.zeros((h, w)) if dense else None
    TO = np.zeros((h, w)) if dense else None
    nms = np.zeros((4, hw, ww)) if debug else None
    tho = np.zeros((hw, ww)) if debug else None
    p10 = np.zeros((10, hw, ww)) if debug else None
    n = lib().subpix_oracle_run_n(_ptr(E), h, w, int(interp_n), float(thresh), float(sigma), float(nbr_radius),
                                  _ptr(th), int(nthreads), _ptr(edges), cap, _ptr(TE), _ptr(TO),
                                  _ptr(nms), _ptr(tho), _ptr(p10))
    out = {"edges": edges[:n].copy()}
    if dense:
        out["TO_E"], out["TO_O"] = TE, TO
    if debug:
        out["nms"], out["theta"], out["planes10"] = nms, tho, p10
    return out


# --------------------------------------------------------------------------
# The reference itself (only where its sources exist: make -C oracle ref)
# --------------------------------------------------------------------------
def ref_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libref_toed.so"))


def ref_lib():
    global _REF
    if _REF is None:
        L = ctypes.CDLL(os.path.join(_HERE, "_ref", "libref_toed.so"))
        L.ref_toed_detect_u8.argtypes = [
            ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, _dp,
            ctypes.c_long, _dp, _dp, _dp]
        L.ref_toed_detect_u8.restype = ctypes.c_long
        L.ref_subpix_to_correct.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
            ctypes.c_double, _dp, ctypes.c_char_p, _dp, ctypes.c_long, _dp, _dp, _dp, _dp]
        L.ref_subpix_to_correct.restype = ctypes.c_long
        L.ref_subpix_to_correct_n.argtypes = [
            _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
            ctypes.c_double, _dp, ctypes.c_char_p, _dp, ctypes.c_long, _dp, _dp]
        L.ref_subpix_to_correct_n.restype = ctypes.c_long
        _REF = L
    return _REF


def ref_detect_u8(img_u8, nthreads: int = 0, planes: bool = False):
    """The reference's ThirdOrderEdgeDetectionCPU<double> at sigma 2 / kernel 17."""
    img = np.ascontiguousarray(img_u8, dtype=np.uint8)
    H, W = img.shape
    cap = 4 * H * W
    edges = np.zeros((cap, 4), np.float64)
    pl = np.zeros((4, 2 * H, 2 * W)) if planes else None
    pm = np.zeros((3, 2 * H, 2 * W)) if planes else None
    t = np.zeros(2)
    nt = nthreads if nthreads > 0 else os.cpu_count()
    with tempfile.TemporaryDirectory() as d:
        n = ref_lib().ref_toed_detect_u8(img.ctypes.data, H, W, nt, d.encode(), _ptr(edges), cap,
                                         _ptr(pl), _ptr(pm), _ptr(t))
    if n < 0:
        raise RuntimeError("reference harness IO error")
    out = {"edges": edges[:n].copy(), "time_conv": t[0], "time_nms": t[1]}
    if planes:
        out["planes"], out["posmaps"] = pl, pm
    return out


def refgpu_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libref_gpu.so"))


_REFGPU = None


def ref_gpu_detect_u8(img_u8, reps: int = 3, device: int = 0, planes: bool = False):
    """The reference's own GPU class ThirdOrderEdgeDetectionGPU<float>
    (sigma 2, kernel 17; gpu_convolve + gpu_nms compiled for sm_103a) on
    one uint8 image.  Returns dict(edges=(N,4) float32, kernel_ms=[...],
    call_ms=[...] [, planes=(4,2H,2W) float32 Ix/Iy/mag/orientation]) --
    per repetition the class's own kernel event times and the wall time of
    its convolve_img + non_maximum_suppresion calls."""
    global _REFGPU
    if _REFGPU is None:
        L = ctypes.CDLL(os.path.join(_HERE, "_ref", "libref_gpu.so"))
        L.ref_gpu_detect_u8.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_long, _dp, ctypes.c_void_p]
        L.ref_gpu_detect_u8.restype = ctypes.c_long
        _REFGPU = L
    img = np.ascontiguousarray(img_u8, dtype=np.uint8)
    H, W = img.shape
    cap = 4 * H * W
    edges = np.zeros((cap, 4), np.float32)
    t = np.zeros(3 * reps)
    pl = np.zeros((4, 2 * H, 2 * W), np.float32) if planes else None
    with tempfile.TemporaryDirectory() as d:
        n = _REFGPU.ref_gpu_detect_u8(img.ctypes.data, H, W, int(device), d.encode(), int(reps),
                                      edges.ctypes.data, cap, _ptr(t), pl.ctypes.data if planes else None)
    if n < 0:
        raise RuntimeError("reference GPU harness IO error")
    t = t.reshape(reps, 3)
    out = {"edges": edges[:n].copy(), "kernel_ms": t[:, 0].tolist(), "call_ms": t[:, 1].tolist()}
    if planes:
        out["planes"] = pl
    return out


def ref_subpix_to_correct(E, thresh=0.1, sigma=2.0, nbr_radius=2.0, theta=None, nthreads=0,
                          dense=False):
    E = np.ascontiguousarray(E, dtype=np.float64)
    h, w = E.shape
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    cap = h * w
    edges = np.zeros((cap, 4))
    TE = np.zeros((h, w)) if dense else None
    TO = np.zeros((h, w)) if dense else None
    tho = np.zeros((h, w))
    times = np.zeros(4)
    nt = nthreads if nthreads > 0 else os.cpu_count()
    with tempfile.TemporaryDirectory() as d:
        n = ref_lib().ref_subpix_to_correct(_ptr(E), h, w, float(thresh), float(sigma), nt,
                                            float(nbr_radius), _ptr(th), d.encode(), _ptr(edges),
                                            cap, _ptr(TE), _ptr(TO), _ptr(tho), _ptr(times))
    out = {"edges": edges[:n].copy(), "theta": tho, "times": times}
    if dense:
        out["TO_E"], out["TO_O"] = TE, TO
    return out


def ref_subpix_to_correct_n(E, interp_n, thresh=0.1, sigma=2.0, nbr_radius=2.0, theta=None, nthreads=0):
    """The reference's SubpixelTOCorrectionCPU<double> at interp_n (dense maps included)."""
    E = np.ascontiguousarray(E, dtype=np.float64)
    h, w = E.shape
    sc = 1 << int(interp_n)
    cap = ((h - 1) * sc + 1) * ((w - 1) * sc + 1)
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
    edges = np.zeros((cap, 4))
    TE, TO = np.zeros((h, w)), np.zeros((h, w))
    nt = nthreads if nthreads > 0 else os.cpu_count()
    with tempfile.TemporaryDirectory() as d:
        n = ref_lib().ref_subpix_to_correct_n(_ptr(E), h, w, int(interp_n), float(thresh), float(sigma), nt,
                                              float(nbr_radius), _ptr(th), d.encode(), _ptr(edges), cap,
                                              _ptr(TE), _ptr(TO))
    return {"edges": edges[:n].copy(), "TO_E": TE, "TO_O": TO}
