"""The header-only C++ drop-in (include/toed_gb300.hpp) used the way the
reference's drivers use ThirdOrderEdgeDetectionGPU<T>, gpu_convolve and
gpu_nms, checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, compare_edgels

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("direct", [False, True])
def test_cpp_shim_matches_oracle(toed, oracle, synth, tmp_path, direct):
    """direct: gpu_convolve built with TOED_GPU_CONVOLVE_DIRECT (the reference
    kernel's full 2-D window sums)."""
    toed.build()
    exe = tmp_path / "shim_driver"
    cuda = "/usr/local/cuda"
    defs = ["-DTOED_GPU_CONVOLVE_DIRECT"] if direct else []
    cmd = ["g++", "-O2", "-std=c++17", *defs, "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
           os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "-o", str(exe),
           toed.LIB_PATH, "-L" + cuda + "/lib64", "-lcudart", "-Wl,-rpath," + os.path.dirname(toed.LIB_PATH),
           "-Wl,-rpath," + cuda + "/lib64"]
    subprocess.run(cmd, check=True)
    H, W = 96, 128
    img = synth.shapes_image(H, W, seed=13).image
    raw = tmp_path / "img.raw"
    raw.write_bytes(img.tobytes())
    r = subprocess.run([str(exe), str(raw), str(H), str(W), str(tmp_path)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    ref = oracle.detect(img.astype(np.float64), 2.0, planes=True)
    e64 = np.fromfile(tmp_path / "edges_f64.bin", dtype=np.float64).reshape(-1, 4)
    e32 = np.fromfile(tmp_path / "edges_f32.bin", dtype=np.float32).reshape(-1, 4)
    assert len(e64) == len(e32) == len(ref["edges"])
    # same order as the reference (row-major over the 2x grid): compare row by row
    m = compare_edgels(ref["edges"], ref["index"], e64, ref["index"])
    assert m["pos_max"] < 1e-3 and m["ori_max"] < 1e-4
    assert np.abs(e32[:, :2] - ref["edges"][:, :2]).max() < 1e-3
    assert (tmp_path / "data_final_output_gpu.txt").exists()
    px = np.fromfile(tmp_path / "posx.bin", dtype=np.float64).reshape(2 * H, 2 * W)
    want = ref["posmaps"][0]
    assert np.array_equal(px != 0, want != 0)
    assert np.abs(px - want).max() < 1e-9


def test_cpp_subpix_shim_matches_oracle(toed, oracle, synth, tmp_path):
    """SubpixelTOCorrectionGPU<T> used as the reference's driver uses
    SubpixelTOCorrectionCPU<T> (main_subpix_to_correction.cpp:279-293):
    estimated orientation (double), a given orientation (float), edgels and
    the dense TO maps against the FP64 oracle."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from test_gpu_subpix import _check
    toed.build()
    exe = tmp_path / "subpix_driver"
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
           os.path.join(ROOT, "tests", "cpp", "subpix_driver.cpp"), "-o", str(exe),
           toed.LIB_PATH, "-L" + cuda + "/lib64", "-lcudart", "-Wl,-rpath," + os.path.dirname(toed.LIB_PATH),
           "-Wl,-rpath," + cuda + "/lib64"]
    subprocess.run(cmd, check=True)
    H, W = 160, 192
    E = synth.ridge_map(H, W, seed=77, n_curves=6).astype(np.float64)
    rng = np.random.default_rng(78)
    theta = rng.uniform(-np.pi, np.pi, (H, W))
    (tmp_path / "E.raw").write_bytes(E.tobytes())
    (tmp_path / "theta.raw").write_bytes(theta.tobytes())
    r = subprocess.run([str(exe), str(tmp_path / "E.raw"), str(H), str(W), str(tmp_path), str(tmp_path / "theta.raw")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)
    ref = oracle.subpix_to_correct(E, 0.1, 2.0, 2.0, dense=True)
    got = np.fromfile(tmp_path / "sp_edges.bin", dtype=np.float64).reshape(-1, 4)
    assert len(ref["edges"]) > 50
    _check(ref["edges"], got)
    te = np.fromfile(tmp_path / "sp_TO_E.bin", dtype=np.float64).reshape(H, W)
    assert np.array_equal(te != 0, ref["TO_E"] != 0)
    assert (tmp_path / "subpix_edges.txt").exists()
    ref2 = oracle.subpix_to_correct(E, 0.1, 2.0, 2.0, theta=theta)
    got2 = np.fromfile(tmp_path / "sp_edges_f32.bin", dtype=np.float32).reshape(-1, 4).astype(np.float64)
    # the float class reads the map rounded to float32: near-tie NMS decisions may differ
    _check(ref2["edges"], got2, agree=0.99, pos=2e-3, ori=2e-3, mag=1e-4)
