"""The reference's own GPU form run on this GPU: its class
ThirdOrderEdgeDetectionGPU<float> with gpu_convolve_kernel and gpu_nms_kernel
compiled unchanged for sm_103a (oracle/_ref/libref_gpu.so, built from the
reference's sources by oracle/Makefile `refgpu`; skipped where they are not
on the host).  Its fixed configuration: sigma 2, kernel 17, uint8 input.

* its edgels against the FP64 oracle with the reference's literal taps: the
  reference's single-image GPU form, computed in FP32, agrees with the
  oracle it is meant to approximate;
* its FP32 Ix / Iy / |grad I| planes against toed_convolve_planes_direct, the
  restatement of its summation (full 2-D window sums, row offset outer)
  given the same literal taps: the restatement that bench.py times beside
  the reference's kernels computes what they compute.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu(oracle):
    if not oracle.refgpu_available():
        if not oracle.ref_sources_present():
            pytest.skip("the reference's sources are not on this host")
        oracle.build(refgpu=True)
    return oracle


def test_reference_gpu_form_vs_oracle_and_restatement(refgpu, toed, synth):
    import torch
    from scipy.spatial import cKDTree
    img = synth.shapes_image(480, 752, seed=1, dtype=np.uint8).image
    H, W = img.shape
    r = refgpu.ref_gpu_detect_u8(img, reps=1, planes=True)
    lit = golden("ref_taps_sigma2")["taps"]
    o = refgpu.detect(img.astype(np.float64), 2.0, 8, tap_block=lit, planes=True)
    assert len(o["edges"]) > 10_000
    # edgel positions: every oracle edgel but a few near-ties has a reference-GPU edgel at its position
    d, _ = cKDTree(r["edges"][:, :2].astype(np.float64)).query(o["edges"][:, :2], k=1)
    assert np.mean(d <= 1e-3) >= 0.995, np.mean(d <= 1e-3)
    assert abs(len(r["edges"]) - len(o["edges"])) <= 0.005 * len(o["edges"])
    # planes: the restatement of the reference kernel's sums, same taps, FP32
    x = torch.as_tensor(img).cuda()
    P = [torch.zeros((2 * H, 2 * W), dtype=torch.float32, device="cuda") for _ in range(4)]
    taps = np.ascontiguousarray(lit, dtype=np.float64)
    st = toed.lib().toed_convolve_planes_direct(
        ctypes.c_void_p(x.data_ptr()), toed.TOED_U8, H, W, W, 2.0, 8, taps.ctypes.data_as(ctypes.c_void_p),
        toed.TOED_F32, *[ctypes.c_void_p(p.data_ptr()) for p in P], ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    for k in range(3):
        mine = P[k].cpu().numpy()
        ref = r["planes"][k]
        scale = np.abs(ref).max()
        assert np.abs(mine - ref).max() <= 1e-6 * scale, (k, np.abs(mine - ref).max() / scale)
