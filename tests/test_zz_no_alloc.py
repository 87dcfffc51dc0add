"""The allocation-free entry point toed_detect_noalloc, called through the C
ABI, must give the same edgels as toed_detect on the same image, on two calls
in a row (the second call reuses the fixed scratch the first one left
behind).

It exists for callers that cannot allocate device memory where they detect
edges (memory owned by a pool or arena, allocation-free real-time loops,
plug-in hosts with pre-sized buffers).  This file is collected last so a
failure here never hides the other tests; it also passes on its own.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(toed, img, out, params):
    import torch
    im = toed.toed_image(img.data_ptr(), img.shape[0], img.shape[1], img.stride(0),
                         toed.TOED_U8 if img.dtype == torch.uint8 else toed.TOED_F32,
                         out["edgels"].data_ptr(), out["capacity"], out["count"].data_ptr(),
                         out["index"].data_ptr())
    s = torch.cuda.current_stream()
    st = toed.lib().toed_detect_noalloc(ctypes.byref(im), ctypes.byref(params), ctypes.c_void_p(s.cuda_stream))
    assert st == toed.TOED_OK, toed.status_string(st)
    s.synchronize()
    n = int(out["count"].item())
    return n, out["edgels"][:n].double().cpu().numpy(), out["index"][:n].cpu().numpy()


@pytest.mark.parametrize("sigma,dtype", [(1.5, np.float32), (2.0, np.uint8)])
def test_noalloc_matches_detect_twice(toed, synth, sigma, dtype):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    toed.build()
    det = toed.Detector(0)
    params = toed.make_params(sigma)
    # two different images so that the second call sees the first call's leftovers
    for seed, (H, W) in [(61, (300, 411)), (62, (257, 190))]:
        img = torch.as_tensor(synth.shapes_image(H, W, seed=seed, dtype=dtype).image).cuda()
        ref = det.detect(img, sigma=sigma)
        out = det.alloc_outputs([(H, W)], capacity=200000, index=True)[0]
        n, e, i = _noalloc(toed, img, out, params)
        assert n == ref["count"] > 50
        # the tolerance of the parity tests; the two entry points run the same kernels
        np.testing.assert_array_equal(i, ref["index"].cpu().numpy())
        np.testing.assert_allclose(e, ref["edgels"].double().cpu().numpy(), rtol=0, atol=1e-4)


@pytest.mark.parametrize("mode", ["fp32", "qad", "f64_out"])
def test_noalloc_modes_match_detect(toed, synth, mode):
    """The precision, orientation and output-dtype branches the entry point
    sets up itself (refine list, QaD ordering pass, 32-byte edgels) against
    toed_detect with the same parameters, two images in a row."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    toed.build()
    det = toed.Detector(0)
    kw = {"fp32": dict(precision=toed.TOED_FP32), "qad": dict(orientation=toed.TOED_ORI_QAD),
          "f64_out": dict(out_dtype=toed.TOED_F64)}[mode]
    params = toed.make_params(1.5, **kw)
    od = kw.get("out_dtype", toed.TOED_F32)
    for seed, (H, W) in [(71, (190, 233)), (72, (141, 260))]:
        img = torch.as_tensor(synth.shapes_image(H, W, seed=seed, dtype=np.float32).image).cuda()
        ref = det.detect(img, sigma=1.5, **kw)
        out = det.alloc_outputs([(H, W)], capacity=100000, out_dtype=od, index=True)[0]
        n, e, i = _noalloc(toed, img, out, params)
        assert n == ref["count"] > 30
        np.testing.assert_array_equal(i, ref["index"].cpu().numpy())
        np.testing.assert_allclose(e, ref["edgels"].double().cpu().numpy(), rtol=0, atol=1e-4)


def test_noalloc_small_capacity_keeps_count(toed, synth):
    """More edgels than the capacity: the call succeeds and the count is the
    exact number of edgels (the list's contents are then undefined)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    toed.build()
    det = toed.Detector(0)
    img = torch.as_tensor(synth.shapes_image(160, 200, seed=73, dtype=np.float32).image).cuda()
    ref = det.detect(img, sigma=1.5)
    assert ref["count"] > 100
    out = det.alloc_outputs([(160, 200)], capacity=37, index=True)[0]
    im = toed.toed_image(img.data_ptr(), 160, 200, 200, toed.TOED_F32, out["edgels"].data_ptr(), 37,
                         out["count"].data_ptr(), out["index"].data_ptr())
    s = torch.cuda.current_stream()
    st = toed.lib().toed_detect_noalloc(ctypes.byref(im), ctypes.byref(toed.make_params(1.5)),
                                        ctypes.c_void_p(s.cuda_stream))
    assert st == toed.TOED_OK
    s.synchronize()
    assert int(out["count"].item()) == ref["count"]


def test_noalloc_rejects_misaligned_float_image(toed):
    """A float32 image pointer that is not 4-byte aligned is refused on the
    host, before any launch, as toed_detect refuses it."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    toed.build()
    buf = torch.zeros(64 * 64 + 4, dtype=torch.float32, device="cuda")
    det = toed.Detector(0)
    out = det.alloc_outputs([(64, 64)], capacity=64, index=True)[0]
    im = toed.toed_image(buf.data_ptr() + 2, 64, 64, 64, toed.TOED_F32, out["edgels"].data_ptr(), 64,
                         out["count"].data_ptr(), None)
    st = toed.lib().toed_detect_noalloc(ctypes.byref(im), ctypes.byref(toed.make_params(1.0)), None)
    assert st == toed.TOED_ERR_INVALID_ARG
    st = toed.lib().toed_detect(det._ctx, ctypes.byref(im), ctypes.byref(toed.make_params(1.0)), None)
    assert st == toed.TOED_ERR_INVALID_ARG


def test_noalloc_rejects_oversize(toed):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    toed.build()
    img = torch.zeros((8, 5000), dtype=torch.float32, device="cuda")
    det = toed.Detector(0)
    out = det.alloc_outputs([(8, 16)], capacity=16, index=True)[0]
    im = toed.toed_image(img.data_ptr(), 8, 5000, 5000, toed.TOED_F32, out["edgels"].data_ptr(), 16,
                         out["count"].data_ptr(), None)
    st = toed.lib().toed_detect_noalloc(ctypes.byref(im), ctypes.byref(toed.make_params(1.0)), None)
    assert st == toed.TOED_ERR_CAPACITY
    im.width = im.pitch = 64
    im.capacity = 10 ** 6
    st = toed.lib().toed_detect_noalloc(ctypes.byref(im), ctypes.byref(toed.make_params(1.0)), None)
    assert st == toed.TOED_ERR_CAPACITY
