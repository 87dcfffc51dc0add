"""The header-only C++ drop-in (include/toed_gb300.hpp) used the way the
reference's drivers use ThirdOrderEdgeDetectionGPU<T>, gpu_convolve and
gpu_nms, checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, compare_edgels

pytestmark = pytest.mark.gpu


def test_cpp_shim_matches_oracle(toed, oracle, synth, tmp_path):
    toed.build()
    exe = tmp_path / "shim_driver"
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
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
