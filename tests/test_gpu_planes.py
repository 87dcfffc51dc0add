"""GPU parity of the compatibility dense-plane path (toed_convolve_planes /
toed_nms_planes, the reference's gpu_convolve / gpu_nms form, and
toed_convolve_planes_direct, the same planes with the reference kernel's
full 2-D window sums) against the oracle's planes."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _planes(toed, img, sigma, dt, direct=False):
    import torch
    H, W = img.shape
    x = torch.as_tensor(img).cuda()
    tdt = torch.float64 if dt == toed.TOED_F64 else torch.float32
    P = [torch.zeros((2 * H, 2 * W), dtype=tdt, device="cuda") for _ in range(4)]
    src_dt = {np.uint8: toed.TOED_U8, np.float32: toed.TOED_F32, np.float64: toed.TOED_F64}[img.dtype.type]
    s = torch.cuda.current_stream().cuda_stream
    conv = toed.lib().toed_convolve_planes_direct if direct else toed.lib().toed_convolve_planes
    st = conv(ctypes.c_void_p(x.data_ptr()), src_dt, H, W, W, float(sigma), 0, None, dt,
              *[ctypes.c_void_p(p.data_ptr()) for p in P], ctypes.c_void_p(s))
    assert st == 0
    pos = [torch.zeros((2 * H, 2 * W), dtype=tdt, device="cuda") for _ in range(2)]
    st = toed.lib().toed_nms_planes(dt, 2 * H, 2 * W, *[ctypes.c_void_p(p.data_ptr()) for p in P[:3]], 2.0, 10,
                                    *[ctypes.c_void_p(p.data_ptr()) for p in pos], ctypes.c_void_p(s))
    assert st == 0
    torch.cuda.synchronize()
    return [p.double().cpu().numpy() for p in P], [p.double().cpu().numpy() for p in pos]


@pytest.mark.parametrize("direct", [False, True])
@pytest.mark.parametrize("sigma", [1.0, 2.0])
def test_planes_f64(detector, toed, oracle, synth, sigma, direct):
    img = synth.shapes_image(70, 90, seed=40, dtype=np.uint8).image
    ref = oracle.detect(img.astype(np.float64), sigma, planes=True)
    P, pos = _planes(toed, img, sigma, toed.TOED_F64, direct)
    for k in range(3):
        scale = np.abs(ref["planes"][k]).max()
        assert np.abs(P[k] - ref["planes"][k]).max() <= 1e-12 * scale
    strong = ref["planes"][2] > 2.0
    d = np.abs(np.angle(np.exp(1j * (P[3] - ref["planes"][3]))))[strong]
    assert d.max() < 1e-9
    mism = (pos[0] != 0) != (ref["posmaps"][0] != 0)
    assert mism.sum() == 0
    both = (pos[0] != 0) & (ref["posmaps"][0] != 0)
    assert np.abs(pos[0][both] - ref["posmaps"][0][both]).max() < 1e-9


@pytest.mark.parametrize("direct", [False, True])
def test_planes_f32(detector, toed, oracle, synth, direct):
    img = synth.shapes_image(70, 90, seed=41, dtype=np.float32).image
    ref = oracle.detect(img.astype(np.float64), 1.5, planes=True)
    P, pos = _planes(toed, img, 1.5, toed.TOED_F32, direct)
    for k in range(3):
        scale = np.abs(ref["planes"][k]).max()
        assert np.abs(P[k] - ref["planes"][k]).max() <= 2e-6 * scale
    both = (pos[0] != 0) & (ref["posmaps"][0] != 0)
    agree = both.sum() / max((pos[0] != 0).sum(), (ref["posmaps"][0] != 0).sum())
    assert agree > 0.999


@pytest.mark.parametrize("radius", [1, 3, 8, 12])
def test_direct_planes_every_radius(detector, toed, oracle, synth, radius):
    """The direct-window kernel is instantiated per radius: FP64 planes equal the
    oracle's at every width, ragged tile edges included (53 x 77)."""
    img = synth.shapes_image(53, 77, seed=42 + radius, dtype=np.float32).image
    sigma = radius / 4.0
    ref = oracle.detect(img.astype(np.float64), sigma, planes=True)
    P, _ = _planes(toed, img, sigma, toed.TOED_F64, direct=True)
    for k in range(3):
        scale = np.abs(ref["planes"][k]).max()
        assert np.abs(P[k] - ref["planes"][k]).max() <= 1e-12 * scale, k
