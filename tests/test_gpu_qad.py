"""GPU parity of the MATLAB quick-and-dirty orientation mode
(TOED_ORI_QAD, third_order_edge_detector.m:91-141) against the oracle's QaD
restatement, through the C ABI.

The mode changes only the emitted orientation: the edgel set, positions and
strengths must equal the grid mode's bit for bit, and the orientation must
meet the same tolerances as the grid mode against its FP64 oracle
(orientation <= 1e-4 rad, wrapped).
"""
import ctypes

import numpy as np
import pytest

from conftest import compare_edgels

pytestmark = pytest.mark.gpu

POS, ORI, STR = 1e-3, 1e-4, 1e-4


def _run(detector, img, sigma, **kw):
    import torch
    x = torch.as_tensor(np.ascontiguousarray(img)).cuda()
    r = detector.detect(x, sigma=sigma, **kw)
    return r["edgels"].double().cpu().numpy(), r["index"].cpu().numpy()


@pytest.mark.parametrize("sigma", [1.0, 1.5, 2.0, 3.0])
@pytest.mark.parametrize("dtype", [np.uint8, np.float32])
def test_qad_vs_oracle(detector, oracle, synth, toed, sigma, dtype):
    img = synth.shapes_image(180, 240, seed=700 + int(sigma * 10) + (dtype == np.uint8), dtype=dtype).image
    ref = oracle.detect(img.astype(np.float64), sigma, orientation="qad")
    eq, iq = _run(detector, img, sigma, orientation=toed.TOED_ORI_QAD)
    eg, ig = _run(detector, img, sigma)
    # only the orientation column differs from the grid mode
    np.testing.assert_array_equal(iq, ig)
    np.testing.assert_array_equal(eq[:, [0, 1, 3]], eg[:, [0, 1, 3]])
    m = compare_edgels(ref["edges"], ref["index"], eq, iq)
    assert m["agreement"] >= 0.999 and m["n_common"] > 50, m
    assert m["pos_max"] <= POS and m["str_rel_max"] <= STR, m
    assert m["ori_max"] <= ORI, m


def test_qad_f64_output_fp32_mode_and_radius(detector, oracle, synth, toed):
    img = synth.shapes_image(120, 160, seed=755, dtype=np.float32).image
    ref = oracle.detect(img.astype(np.float64), 2.0, orientation="qad")
    for kw in ({"out_dtype": toed.TOED_F64}, {"precision": toed.TOED_FP32}):
        e, i = _run(detector, img, 2.0, orientation=toed.TOED_ORI_QAD, **kw)
        m = compare_edgels(ref["edges"], ref["index"], e, i)
        assert m["agreement"] >= 0.999 and m["pos_max"] <= POS and m["ori_max"] <= ORI, (kw, m)
    # an explicit radius other than ceil(4 sigma)
    ref = oracle.detect(img.astype(np.float64), 1.5, 5, orientation="qad")
    e, i = _run(detector, img, 1.5, radius=5, orientation=toed.TOED_ORI_QAD)
    m = compare_edgels(ref["edges"], ref["index"], e, i)
    assert m["agreement"] >= 0.999 and m["ori_max"] <= ORI, m


def test_qad_batch_equals_single_and_noalloc(detector, synth, toed):
    import torch
    sizes = [(64, 100), (200, 47), (257, 129), (90, 301)]
    imgs = [torch.as_tensor(synth.shapes_image(h, w, seed=780 + k, dtype=np.float32).image).cuda()
            for k, (h, w) in enumerate(sizes)]
    res = detector.detect_batch(imgs, sigma=1.5, orientation=toed.TOED_ORI_QAD)
    params = toed.make_params(1.5, orientation=toed.TOED_ORI_QAD)
    for im, r in zip(imgs, res):
        s = detector.detect(im, sigma=1.5, orientation=toed.TOED_ORI_QAD)
        assert torch.equal(s["edgels"], r["edgels"]) and torch.equal(s["index"], r["index"])
        out = detector.alloc_outputs([tuple(im.shape)], capacity=100000, index=True)[0]
        st = toed.lib().toed_detect_noalloc(
            ctypes.byref(toed.toed_image(im.data_ptr(), im.shape[0], im.shape[1], im.stride(0), toed.TOED_F32,
                                         out["edgels"].data_ptr(), out["capacity"], out["count"].data_ptr(),
                                         out["index"].data_ptr())),
            ctypes.byref(params), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == toed.TOED_OK
        torch.cuda.synchronize()
        n = int(out["count"].item())
        assert n == r["count"]
        assert torch.equal(out["index"][:n], r["index"])
        assert torch.allclose(out["edgels"][:n], r["edgels"], rtol=0, atol=1e-4)


def test_qad_host_batch(detector, synth, toed):
    import torch
    sizes = [(96, 128), (150, 77), (64, 300)]
    imgs = [torch.as_tensor(synth.shapes_image(h, w, seed=790 + k, dtype=np.float32).image)
            for k, (h, w) in enumerate(sizes)]
    params = toed.make_params(2.0, orientation=toed.TOED_ORI_QAD)
    outs = detector.alloc_host_outputs(sizes, index=True)
    detector.detect_host([im.pin_memory() for im in imgs], outs, params, chunks=2)
    for im, o in zip(imgs, outs):
        d = detector.detect(im.cuda(), sigma=2.0, orientation=toed.TOED_ORI_QAD)
        n = int(o["count"].item())
        assert n == d["count"]
        assert torch.equal(o["edgels"][:n], d["edgels"].cpu()) and torch.equal(o["index"][:n], d["index"].cpu())


def test_qad_argument_checks(detector, toed):
    import torch
    img = torch.zeros((32, 32), dtype=torch.float32, device="cuda")
    out = detector.alloc_outputs([(32, 32)], capacity=16, index=True)[0]
    im = toed.toed_image(img.data_ptr(), 32, 32, 32, toed.TOED_F32, out["edgels"].data_ptr(), 16,
                         out["count"].data_ptr(), out["index"].data_ptr())
    bad = toed.make_params(2.0, orientation=2)
    assert toed.lib().toed_detect_batch(detector._ctx, ctypes.byref(im), 1, ctypes.byref(bad), None) == \
        toed.TOED_ERR_INVALID_ARG
    # the adjoint is that of the grid-point orientation only
    g = toed.toed_grad_image(img.data_ptr(), 32, 32, 32, toed.TOED_F32, 0, None, None, img.data_ptr())
    gs = ctypes.c_double(0.0)
    st = toed.lib().toed_backward_batch(detector._ctx, ctypes.byref(g), 1,
                                        ctypes.byref(toed.make_params(2.0, orientation=toed.TOED_ORI_QAD)),
                                        ctypes.addressof(gs), None)
    assert st == toed.TOED_ERR_UNSUPPORTED
