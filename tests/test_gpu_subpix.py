"""GPU parity of the subpixel TO-correction path
(toed_subpix_to_correct_batch) against the reference's golden fixtures and
the FP64 oracle.  Edgels are matched by their pixel (round of the NMS
position is not used: each pixel holds at most one edgel, identified by the
truncated subpixel position's nearest source pixel)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, wrap_angle

pytestmark = pytest.mark.gpu

SUBPIX_CASES = sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "subpix_*.npz")))


def _match(ref, got, tol=0.05):
    """Greedy match by position (edgels of one map are > 0.1 px apart
    unless they come from neighbouring pixels)."""
    if len(ref) == 0 or len(got) == 0:
        return np.zeros(0, int), np.zeros(0, int)
    from scipy.spatial import cKDTree
    tr = cKDTree(got[:, :2])
    d, j = tr.query(ref[:, :2], k=1)
    ok = d < tol
    return np.flatnonzero(ok), j[ok]


def _check(ref, got, agree=0.999, pos=1e-3, ori=1e-4, mag=1e-4):
    ia, ib = _match(ref, got)
    n = max(len(ref), len(got))
    a = len(ia) / n if n else 1.0
    assert a >= agree, (a, len(ref), len(got))
    if len(ia):
        pe = np.hypot(*(ref[ia, :2] - got[ib, :2]).T).max()
        oe = wrap_angle(ref[ia, 2] - got[ib, 2]).max()
        me = (np.abs(ref[ia, 3] - got[ib, 3]) / np.maximum(np.abs(ref[ia, 3]), 1e-12)).max()
        assert pe <= pos and oe <= ori and me <= mag, (pe, oe, me)
    return a


def _run(detector, E, thresh, sigma, rad, theta=None, **kw):
    import torch
    t = torch.as_tensor(np.ascontiguousarray(E)).cuda()
    th = None if theta is None else [torch.as_tensor(np.ascontiguousarray(theta)).cuda()]
    r = detector.subpix_to_correct_batch([t], thresh=thresh, sigma=sigma, nbr_radius=rad, thetas=th, **kw)[0]
    return r


@pytest.mark.parametrize("case", SUBPIX_CASES)
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_golden(detector, toed, case, dt):
    g = golden("subpix_" + case)
    thresh, sigma, rad = g["params"][:3]
    interp_n = int(g["params"][3]) if len(g["params"]) > 3 else 0
    th = g["theta_in"].astype(dt) if "theta_in" in g else None
    r = _run(detector, g["E"].astype(dt), thresh, sigma, rad, theta=th, out_dtype=toed.TOED_F64,
             interp_n=interp_n)
    got = r["edgels"].cpu().numpy()
    assert r["count"] == len(got)
    # a float32 map is not the reference's map: its rounding moves the edgels themselves
    _check(g["edges"], got, ori=1e-4 if dt == np.float64 else 1e-3)
    # dense maps: same support up to the few edgels that moved across a rounding boundary
    TE = r["TO_E"].cpu().numpy()
    assert ((TE != 0) != (g["TO_E"] != 0)).sum() <= max(2, 0.002 * (g["TO_E"] != 0).sum())


@pytest.mark.parametrize("seed,H,W,sigma,thresh,est", [(7, 200, 260, 2.0, 0.1, True), (8, 150, 333, 1.5, 0.15, False),
                                                        (9, 64, 64, 1.0, 0.2, True)])
def test_vs_oracle(detector, oracle, synth, toed, seed, H, W, sigma, thresh, est):
    E = synth.ridge_map(H, W, seed=seed, n_curves=6).astype(np.float32)
    th = None if est else np.random.default_rng(seed).uniform(-3, 3, E.shape).astype(np.float32)
    ref = oracle.subpix_to_correct(E.astype(np.float64), thresh, sigma, 2.0,
                                   theta=None if th is None else th.astype(np.float64))
    r = _run(detector, E, thresh, sigma, 2.0, theta=th, out_dtype=toed.TOED_F64)
    # a random per-pixel orientation field (est False) makes the correction
    # vector nearly cancel at a few edgels, where the FP32 planes' rounding
    # reaches the angle multiplied by that cancellation: 2e-4 rad there
    _check(ref["edges"], r["edgels"].cpu().numpy(), ori=1e-4 if est else 2e-4)


def test_batch_and_fp32_mode(detector, oracle, synth, toed):
    import torch
    maps = [synth.ridge_map(h, w, seed=50 + h, n_curves=5).astype(np.float32) for h, w in [(96, 128), (130, 70), (64, 200)]]
    res = detector.subpix_to_correct_batch([torch.as_tensor(m).cuda() for m in maps], thresh=0.1, sigma=2.0,
                                           nbr_radius=2.0, out_dtype=toed.TOED_F64)
    for m, r in zip(maps, res):
        ref = oracle.subpix_to_correct(m.astype(np.float64), 0.1, 2.0, 2.0)
        _check(ref["edges"], r["edgels"].cpu().numpy())
    r32 = detector.subpix_to_correct_batch([torch.as_tensor(maps[0]).cuda()], thresh=0.1, sigma=2.0,
                                           nbr_radius=2.0, precision=toed.TOED_FP32)[0]
    ref = oracle.subpix_to_correct(maps[0].astype(np.float64), 0.1, 2.0, 2.0)
    _check(ref["edges"], r32["edgels"].double().cpu().numpy(), ori=2e-3, mag=1e-3)


@pytest.mark.parametrize("interp_n,est", [(1, True), (2, False)])
def test_work_grid_vs_oracle(detector, oracle, synth, toed, interp_n, est):
    """interp_n > 0: the map (and orientation) resized onto the 2^n work grid."""
    E = synth.ridge_map(90, 110, seed=60 + interp_n, n_curves=5).astype(np.float32)
    th = None if est else np.random.default_rng(61).uniform(0, 3, E.shape).astype(np.float32)
    ref = oracle.subpix_to_correct(E.astype(np.float64), 0.1, 2.0, 2.0,
                                   theta=None if th is None else th.astype(np.float64), dense=True,
                                   interp_n=interp_n)
    r = _run(detector, E, 0.1, 2.0, 2.0, theta=th, out_dtype=toed.TOED_F64, interp_n=interp_n)
    assert len(ref["edges"]) > 100
    _check(ref["edges"], r["edgels"].cpu().numpy())
    TE = r["TO_E"].cpu().numpy()
    assert TE.shape == E.shape
    assert ((TE != 0) != (ref["TO_E"] != 0)).sum() <= max(2, 0.002 * (ref["TO_E"] != 0).sum())
