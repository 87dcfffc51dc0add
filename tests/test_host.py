"""CPU-only tests: the C ABI library builds for sm_103a, loads without a GPU
and exports every symbol include/toed_gb300.h declares; the ctypes mirror of
the ABI structs matches the C layout; host-side helpers behave."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "toed_gb300.h")


def _declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(toed_[a-z_0-9]+)\s*\(", src)))


def test_library_builds_and_exports_header_symbols(toed):
    path = toed.build()
    assert os.path.exists(path)
    L = ctypes.CDLL(path)
    decl = _declared_functions()
    assert len(decl) >= 11
    for name in decl:
        assert hasattr(L, name), name
    assert sorted(toed.C_SYMBOLS) == sorted(n for n in decl if n in toed.C_SYMBOLS)
    assert set(decl) <= set(toed.C_SYMBOLS) | set(getattr(toed, "C_SYMBOLS_EXTRA", []))


def test_status_strings(toed):
    toed.build()
    L = toed.lib()
    for s in range(7):
        assert toed.status_string(s)
    assert L.toed_status_string(99).decode() == "unknown status"
    p = toed.toed_params()
    L.toed_params_default(ctypes.byref(p), ctypes.c_float(2.0))
    assert (p.sigma, p.radius, p.threshold, p.border) == (2.0, 0, 2.0, 10)
    assert (p.orientation, p.nms_direction) == (toed.TOED_ORI_GRID, toed.TOED_NMS_GRADIENT)


def test_struct_layout_matches_header(toed, tmp_path):
    c = tmp_path / "layout.c"
    c.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "toed_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(toed_image), offsetof(toed_image, dtype),
         offsetof(toed_image, edgels), offsetof(toed_image, capacity), offsetof(toed_image, count),
         offsetof(toed_image, grid_index), sizeof(toed_params), offsetof(toed_params, precision),
         offsetof(toed_params, orientation), sizeof(toed_tuning), sizeof(toed_host_image),
         offsetof(toed_host_image, grid_index), sizeof(toed_edgemap), sizeof(toed_subpix_params),
         offsetof(toed_params, nms_direction));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include", str(c), "-o",
                    str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    T, P, HI = toed.toed_image, toed.toed_params, toed.toed_host_image
    want = [ctypes.sizeof(T), T.dtype.offset, T.edgels.offset, T.capacity.offset, T.count.offset,
            T.grid_index.offset, ctypes.sizeof(P), P.precision.offset, P.orientation.offset,
            ctypes.sizeof(toed.toed_tuning), ctypes.sizeof(HI), HI.grid_index.offset,
            ctypes.sizeof(toed.toed_edgemap), ctypes.sizeof(toed.toed_subpix_params), P.nms_direction.offset]
    assert got == want


def test_no_cpu_fallback(toed, monkeypatch):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        toed.Detector(0)


def test_synth_deterministic(synth):
    a = synth.shapes_image(60, 80, seed=3).image
    b = synth.shapes_image(60, 80, seed=3).image
    assert a.dtype == np.uint8 and np.array_equal(a, b)
    f = synth.shapes_image(60, 80, seed=3, dtype=np.float32).image
    assert f.dtype == np.float32 and f.min() >= 0 and f.max() <= 255
    sizes = synth.uneven_batch_shapes()
    assert len(sizes) == 64 and all(h % 4 == 0 and w % 4 == 0 and 256 <= h <= 2048 for h, w in sizes)
    E = synth.ridge_map(64, 64, seed=1, n_curves=3)
    assert E.min() >= 0 and E.max() <= 1


def test_ellipse_distance(synth):
    e = synth.Ellipse(10.0, 20.0, 8.0, 3.0, 0.3, 100.0)
    t = np.linspace(0, 2 * np.pi, 50)
    c, s = np.cos(e.theta), np.sin(e.theta)
    bx = e.cx + e.a * np.cos(t) * c - e.b * np.sin(t) * s
    by = e.cy + e.a * np.cos(t) * s + e.b * np.sin(t) * c
    assert np.abs(synth.ellipse_distance(bx, by, e)).max() < 1e-9
    assert abs(synth.ellipse_distance(np.array([10.0]), np.array([20.0]), e)[0] - 3.0) < 1e-9


def test_cpp_dropin_header_and_drivers_compile(toed, tmp_path):
    """The header-only C++ drop-in (both classes and the free functions) and
    the reference-style drivers that exercise it compile and link here."""
    toed.build()
    for drv, defs in (("shim_driver.cpp", []), ("shim_driver.cpp", ["-DTOED_GPU_CONVOLVE_DIRECT"]),
                      ("subpix_driver.cpp", [])):
        exe = tmp_path / (drv.replace(".cpp", "") + ("_direct" if defs else ""))
        subprocess.run(["g++", "-O1", "-std=c++17", "-Wall", *defs, "-I" + os.path.join(ROOT, "include"),
                        "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "cpp", drv), "-o", str(exe),
                        toed.LIB_PATH, "-L/usr/local/cuda/lib64", "-lcudart"], check=True)
        assert exe.exists()


def test_batch_driver_cli_without_gpu(toed, tmp_path):
    """toed_batch is built by build(); its usage text and input checks need
    no GPU."""
    toed.build()
    exe = os.path.join(os.path.dirname(toed.LIB_PATH), "toed_batch")
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "edges_gpu.txt" in r.stdout
    r = subprocess.run([exe, str(tmp_path / "missing"), str(tmp_path / "out")], capture_output=True, text=True)
    assert r.returncode == 1 and "not found" in r.stderr
    r = subprocess.run([exe, str(tmp_path), str(tmp_path / "out"), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown option" in r.stderr
