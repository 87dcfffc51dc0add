"""Bounds-checked build (-DTOED_DEBUG_BOUNDS; compute-sanitizer is not
available on the GPU hosts): the detection kernel's guarded shared- and
global-memory indices are checked at run time and a failure is reported as
TOED_FLAG_BOUNDS (the access is skipped; nothing traps).  Small odd-sized
cases -- sizes below one tile, widths that are not multiples of 4 or 8, thin
and single-pixel images, every staging mode, several radii, the
corrected-normal mode -- run through the debug library in a process of its
own; no check may fail and the edgels must equal the release library's."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(37, 53), (1, 1), (3, 200), (200, 3), (15, 31), (61, 129), (130, 97), (257, 190)]

CHILD = r"""
import json, os, sys
sys.path.insert(0, {tests!r})
from conftest import load_package
toed = load_package()
import importlib, numpy as np, torch
synth = importlib.import_module("toed_gb300.synth")
det = toed.Detector(0)
cases = {cases!r}
out = []
for sigma in (0.5, 1.5, 2.0):
    for nd in (0, 1):
        for staging in ("tma", "async", "plain"):
            p = toed.make_params(sigma, nms_direction=nd)
            det.set_tuning(p, 14 if staging != "tma" else 30, staging)
            ims = [torch.as_tensor(synth.shapes_image(h, w, seed=900 + k, n_shapes=4, radius_range=(3, 40),
                                                      dtype=np.float32 if k % 2 else np.uint8).image).cuda()
                   for k, (h, w) in enumerate(cases)]
            res = det.detect_batch(ims, sigma=sigma, nms_direction=nd)
            out.append({{"sigma": sigma, "nms": nd, "staging": staging, "flags": det.flags(),
                        "counts": [r["count"] for r in res],
                        "edgels": [r["edgels"].double().cpu().numpy().tolist() for r in res]}})
print("RESULT " + json.dumps(out))
"""


def _run(lib_path):
    code = CHILD.format(tests=os.path.dirname(os.path.abspath(__file__)), cases=CASES)
    env = dict(os.environ, TOED_LIBRARY=lib_path)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    line = [l for l in r.stdout.splitlines() if l.startswith("RESULT ")][-1]
    return json.loads(line[7:])


def test_bounds_checked_build_small_odd_sizes(toed):
    dbg = toed.build(debug=True)
    got = _run(dbg)
    ref = _run(toed.LIB_PATH)
    assert len(got) == len(ref) == 18
    for g, r in zip(got, ref):
        assert g["flags"] & toed.TOED_FLAG_BOUNDS == 0, g["flags"]
        assert g["flags"] == r["flags"] == 0
        assert g["counts"] == r["counts"]
        for a, b in zip(g["edgels"], r["edgels"]):
            np.testing.assert_allclose(np.array(a).reshape(-1, 4), np.array(b).reshape(-1, 4), rtol=0, atol=1e-5,
                                       equal_nan=True)
    assert sum(sum(g["counts"]) for g in got) > 1000
