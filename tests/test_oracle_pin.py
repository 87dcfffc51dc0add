"""Pins the CPU oracle (oracle/toed_oracle.c) to the reference.

* Against committed golden fixtures produced by the reference's own
  ThirdOrderEdgeDetectionCPU<double> / SubpixelTOCorrectionCPU<double>
  (tests/golden/make_golden.py): bit-identical given the reference's literal
  taps, and within 1e-10 with taps from the formula.
* Against the reference compiled here (oracle/_ref), when its sources exist,
  on extra seeded images.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden

TOED_CASES = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "toed_*.npz")))
SUBPIX_CASES = sorted(os.path.basename(p)[7:-4] for p in glob.glob(os.path.join(GOLDEN, "subpix_*.npz")))


def test_fixtures_present():
    assert len(TOED_CASES) >= 10 and len(SUBPIX_CASES) >= 3


def test_literal_taps_match_formula(oracle):
    lit = golden("ref_taps_sigma2")["taps"]
    f = oracle.taps(2.0, 8)
    assert lit.shape == f.shape == (8, 19)
    assert np.max(np.abs(lit - f)) < 1e-15


@pytest.mark.parametrize("case", TOED_CASES)
def test_toed_bit_exact_with_reference_taps(oracle, case):
    g = golden("toed_" + case)
    lit = golden("ref_taps_sigma2")["taps"]
    o = oracle.detect(g["image"].astype(np.float64), 2.0, 8, tap_block=lit, planes="planes" in g)
    assert o["edges"].shape == g["edges"].shape
    assert np.array_equal(o["edges"], g["edges"], equal_nan=True)
    if "planes" in g:
        assert np.array_equal(o["planes"], g["planes"], equal_nan=True)


@pytest.mark.parametrize("case", TOED_CASES)
def test_toed_formula_taps_close(oracle, case):
    g = golden("toed_" + case)
    o = oracle.detect(g["image"].astype(np.float64), 2.0)
    assert o["edges"].shape == g["edges"].shape
    if len(g["edges"]):
        assert np.nanmax(np.abs(o["edges"] - g["edges"])) < 1e-10


def test_toed_known_answers(oracle):
    # vertical 50 -> 150 step between columns 31 | 32: with the (k-1)/2
    # output convention (cpu_toed.cpp:516) the edge reports x = 31.0,
    # orientation -pi/2 (atan2(TO_Ix, -TO_Iy), cpu_toed.cpp:232)
    g = golden("toed_step_v")
    e = g["edges"]
    assert len(e) > 0
    assert np.allclose(e[:, 0], 31.0, atol=3e-3)  # zero padding bends it near the top/bottom
    assert np.allclose(e[:, 2], -np.pi / 2, atol=1e-2)
    assert np.allclose(e[:, 3], 20.1, atol=0.1)
    assert len(golden("toed_constant")["edges"]) == 0
    assert len(golden("toed_tiny_8x9")["edges"]) == 0
    # disc of radius 20 at (39.3, 35.7): edgels lie near the circle (the
    # output is the true position - 0.5 px)
    d = golden("toed_disc")["edges"]
    r = np.hypot(d[:, 0] + 0.5 - 39.3, d[:, 1] + 0.5 - 35.7)
    assert np.median(np.abs(r - 20.0)) < 0.6


@pytest.mark.parametrize("case", SUBPIX_CASES)
def test_subpix_bit_exact(oracle, case):
    g = golden("subpix_" + case)
    thresh, sigma, rad = g["params"][:3]
    interp_n = int(g["params"][3]) if len(g["params"]) > 3 else 0
    th = g["theta_in"] if "theta_in" in g else None
    o = oracle.subpix_to_correct(g["E"], thresh, sigma, rad, theta=th, dense=True, interp_n=interp_n)
    assert np.array_equal(o["edges"], g["edges"], equal_nan=True)
    assert np.array_equal(o["TO_E"], g["TO_E"])
    assert np.array_equal(o["TO_O"], g["TO_O"])


def _ref_or_skip(oracle):
    if not oracle.ref_available():
        if oracle.ref_sources_present():
            oracle.build(ref=True)
        else:
            pytest.skip("reference sources not present")


@pytest.mark.parametrize("seed,H,W", [(101, 40, 57), (102, 77, 64), (103, 120, 90)])
def test_toed_live_reference(oracle, synth, seed, H, W):
    _ref_or_skip(oracle)
    img = synth.shapes_image(H, W, seed=seed, noise_std=4.0).image
    r = oracle.ref_detect_u8(img, planes=True)
    lit = golden("ref_taps_sigma2")["taps"]
    o = oracle.detect(img.astype(np.float64), 2.0, 8, tap_block=lit, planes=True)
    assert np.array_equal(r["edges"], o["edges"], equal_nan=True)
    assert np.array_equal(r["planes"], o["planes"], equal_nan=True)
    assert np.array_equal(r["posmaps"], o["posmaps"], equal_nan=True)


@pytest.mark.parametrize("seed,est", [(201, True), (202, False)])
def test_subpix_live_reference(oracle, synth, seed, est):
    _ref_or_skip(oracle)
    E = synth.ridge_map(70, 88, seed=seed, n_curves=4).astype(np.float64)
    th = None if est else np.random.default_rng(seed).uniform(0, np.pi, E.shape)
    r = oracle.ref_subpix_to_correct(E, 0.12, 1.5, 2.0, theta=th, dense=True)
    o = oracle.subpix_to_correct(E, 0.12, 1.5, 2.0, theta=th, dense=True, debug=True)
    assert np.array_equal(r["edges"], o["edges"], equal_nan=True)
    assert np.array_equal(r["TO_E"], o["TO_E"]) and np.array_equal(r["TO_O"], o["TO_O"])
    assert np.array_equal(r["theta"], o["theta"])


@pytest.mark.parametrize("interp_n", [1, 2])
def test_subpix_live_reference_interp(oracle, synth, interp_n):
    """interp_n > 0: the reference resizes the map onto the 2^n work grid."""
    _ref_or_skip(oracle)
    E = synth.ridge_map(44, 52, seed=300 + interp_n, n_curves=3).astype(np.float64)
    r = oracle.ref_subpix_to_correct_n(E, interp_n, 0.1, 2.0, 2.0)
    o = oracle.subpix_to_correct(E, 0.1, 2.0, 2.0, dense=True, interp_n=interp_n)
    assert len(r["edges"]) > 20
    assert np.array_equal(r["edges"], o["edges"], equal_nan=True)
    assert np.array_equal(r["TO_E"], o["TO_E"]) and np.array_equal(r["TO_O"], o["TO_O"])


@pytest.mark.parametrize("sigma", [1.5, 2.0])
@pytest.mark.parametrize("dtype", [np.uint8, np.float32])
def test_frozen_matches_oracle(oracle, synth, sigma, dtype):
    """The adjoint's FP64 reference (oracle/frozen.py, torch FP64 with the
    selection frozen) evaluated at the C oracle's own edgels gives the C
    oracle's [x, y, orientation, strength] -- so the reference gradient
    differentiates the same function the oracle (pinned bit for bit to the
    reference above) computes."""
    import torch
    from oracle import frozen
    img = synth.shapes_image(160, 200, seed=77, n_shapes=14, noise_std=4.0, dtype=dtype).image.astype(np.float64)
    o = oracle.detect(img, sigma)
    assert len(o["index"]) > 1000
    r = oracle.default_radius(sigma)
    with torch.no_grad():
        f = frozen.edgel_outputs(torch.as_tensor(img), torch.tensor(sigma, dtype=torch.float64),
                                 torch.as_tensor(o["index"]), r).numpy()
    e = o["edges"]
    assert np.max(np.abs(f[:, :2] - e[:, :2])) <= 1e-12
    assert np.max(np.abs(f[:, 3] - e[:, 3]) / np.abs(e[:, 3])) <= 1e-12
    d = np.abs(np.angle(np.exp(1j * (f[:, 2] - e[:, 2]))))
    assert np.nanmax(d) <= 1e-12
    assert np.array_equal(np.isnan(f[:, 2]), np.isnan(e[:, 2]))
