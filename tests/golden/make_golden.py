"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a container where the reference sources exist (it builds
oracle/_ref/libref_toed.so from them with ``make -C oracle ref``):

    python tests/golden/make_golden.py [--ref-dir /path/to/reference]

Fixtures (all .npz):
* ``ref_taps_sigma2``  -- the reference's literal tap table (cpu_toed.cpp:150-167),
  read from its source text, 8 x 19 in the order G, Gx, Gxx, Gxxx, G_sh,
  Gx_sh, Gxx_sh, Gxxx_sh.  Used to show the oracle reproduces the reference
  bit for bit when given the same taps.
* ``toed_<case>``      -- input image (uint8), the reference's edgel list
  (FP64, N x 4) from ThirdOrderEdgeDetectionCPU<double> at sigma 2 / kernel 17,
  and for small cases its Ix / Iy / |grad| / orientation planes.
* ``subpix_<case>``    -- edge map, optional orientation, the reference's
  SubpixelTOCorrectionCPU<double> edgel list and dense TO maps; the
  ``_n1`` / ``_n2`` cases run it on the 2^n work grid (interp_n = 1, 2) and
  store interp_n as the fourth parameter.

``--only PREFIX`` regenerates just the fixtures whose name starts with PREFIX.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)


def _synth():
    import importlib.util
    p = os.path.join(ROOT, "third-order-edge-detector_gb300", "synth.py")
    spec = importlib.util.spec_from_file_location("toed_synth_fixture", p)
    m = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = m
    spec.loader.exec_module(m)
    return m


TAP_NAMES = ["G_of_x", "Gx", "Gxx", "Gxxx", "G_of_x_sh", "Gx_sh", "Gxx_sh", "Gxxx_sh"]


def literal_taps(ref_dir: str) -> np.ndarray:
    src = open(os.path.join(ref_dir, "cpu_toed.cpp")).read()
    rows = []
    for n in TAP_NAMES:
        m = re.search(r"T\s+%s\[\]\s*=\s*\{([^}]*)\}" % re.escape(n), src)
        rows.append([float(v) for v in m.group(1).split(",")])
    return np.array(rows, np.float64)


def kat_images():
    out = {}
    step = np.full((64, 64), 50, np.uint8)
    step[:, 32:] = 150
    out["step_v"] = step
    out["step_h"] = np.ascontiguousarray(step.T)
    out["constant"] = np.full((48, 40), 77, np.uint8)
    yy, xx = np.mgrid[0:72, 0:80]
    disc = np.where((xx - 39.3) ** 2 + (yy - 35.7) ** 2 <= 20.0 ** 2, 200, 40).astype(np.uint8)
    out["disc"] = disc
    out["tiny_8x9"] = (np.arange(72).reshape(8, 9) * 3).astype(np.uint8)
    out["thin_12x200"] = np.tile(np.where(np.arange(200) % 50 < 25, 30, 220).astype(np.uint8), (12, 1))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=os.environ.get("TOED_REF_DIR") or subprocess.run(
        ["make", "-s", "-C", os.path.join(ROOT, "oracle"), "refdir"], capture_output=True, text=True).stdout.strip(),
        help="reference checkout (default: $TOED_REF_DIR, else the oracle recipe's default)")
    ap.add_argument("--only", default="", help="regenerate only fixtures whose name starts with this")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_DIR={args.ref_dir}"],
                   check=True)
    import oracle
    synth = _synth()

    def want(name):
        return name.startswith(args.only)

    if want("ref_taps_sigma2"):
        np.savez_compressed(os.path.join(HERE, "ref_taps_sigma2.npz"), taps=literal_taps(args.ref_dir))

    cases = dict(kat_images())
    cases["shapes_37x53"] = synth.shapes_image(37, 53, seed=11).image
    cases["shapes_64x80"] = synth.shapes_image(64, 80, seed=12).image
    cases["shapes_96x128"] = synth.shapes_image(96, 128, seed=13).image
    cases["shapes_150x97"] = synth.shapes_image(150, 97, seed=14, noise_std=6.0).image
    cases["shapes_752x480"] = synth.shapes_image(480, 752, seed=1).image
    for name, img in cases.items():
        if not want(f"toed_{name}"):
            continue
        small = img.size <= 64 * 64
        r = oracle.ref_detect_u8(img, planes=small)
        d = {"image": img, "edges": r["edges"]}
        if small:
            d["planes"] = r["planes"]
        np.savez_compressed(os.path.join(HERE, f"toed_{name}.npz"), **d)
        print(f"toed_{name}: {img.shape} -> {len(r['edges'])} edgels")

    sub = {
        "ridges_96x120_est": (synth.ridge_map(96, 120, seed=21, n_curves=5), None, 0.1, 2.0, 2.0),
        "ridges_128x160_theta": (synth.ridge_map(128, 160, seed=22, n_curves=6),
                                 np.random.Generator(np.random.PCG64(23)).uniform(-4, 4, (128, 160)),
                                 0.1, 2.0, 2.0),
        "ridges_80x90_s15_r0": (synth.ridge_map(80, 90, seed=24, n_curves=4), None, 0.15, 1.5, 0.0),
    }
    for name, (E, th, thresh, sigma, rad) in sub.items():
        if not want(f"subpix_{name}"):
            continue
        E = E.astype(np.float64)
        r = oracle.ref_subpix_to_correct(E, thresh, sigma, rad, theta=th, dense=True)
        d = {"E": E, "edges": r["edges"], "TO_E": r["TO_E"], "TO_O": r["TO_O"], "theta": r["theta"],
             "params": np.array([thresh, sigma, rad])}
        if th is not None:
            d["theta_in"] = th
        np.savez_compressed(os.path.join(HERE, f"subpix_{name}.npz"), **d)
        print(f"subpix_{name}: {E.shape} -> {len(r['edges'])} edgels")

    # the 2^n work grid (interp_n > 0): bilinear resize, scaled margin, positions / 2^n
    sub_n = {
        "ridges_60x72_est_n1": (synth.ridge_map(60, 72, seed=25, n_curves=4), None, 0.1, 2.0, 2.0, 1),
        "ridges_48x56_theta_n2": (synth.ridge_map(48, 56, seed=26, n_curves=3),
                                  np.random.Generator(np.random.PCG64(27)).uniform(0, 3, (48, 56)),
                                  0.1, 1.5, 2.0, 2),
    }
    for name, (E, th, thresh, sigma, rad, n) in sub_n.items():
        if not want(f"subpix_{name}"):
            continue
        E = E.astype(np.float64)
        r = oracle.ref_subpix_to_correct_n(E, n, thresh, sigma, rad, theta=th)
        d = {"E": E, "edges": r["edges"], "TO_E": r["TO_E"], "TO_O": r["TO_O"],
             "params": np.array([thresh, sigma, rad, n])}
        if th is not None:
            d["theta_in"] = th
        np.savez_compressed(os.path.join(HERE, f"subpix_{name}.npz"), **d)
        print(f"subpix_{name}: {E.shape} (interp_n {n}) -> {len(r['edges'])} edgels")


if __name__ == "__main__":
    main()
