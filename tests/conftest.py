"""Shared test fixtures: package loader, the ``gpu`` marker, parity metrics.

The package directory ``third-order-edge-detector_gb300/`` is not a valid
Python identifier; it is registered as the importable name ``toed_gb300``.
"""
from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG_DIR = os.path.join(ROOT, "third-order-edge-detector_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    name = "toed_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def toed():
    return load_package()


@pytest.fixture(scope="session")
def synth():
    load_package()
    import importlib
    return importlib.import_module("toed_gb300.synth")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def detector(toed):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    toed.build()
    return toed.Detector(0)


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def wrap_angle(d):
    return np.abs(np.angle(np.exp(1j * d)))


def compare_edgels(ref_edges, ref_index, got_edges, got_index):
    """Edgel-set agreement (match by 2x-grid index) and errors on the matched
    set: position (px), orientation (rad, wrapped), relative strength."""
    ref_index = np.asarray(ref_index, np.int64)
    got_index = np.asarray(got_index, np.int64)
    common, ia, ib = np.intersect1d(ref_index, got_index, return_indices=True)
    denom = max(len(ref_index), len(got_index))
    out = {
        "n_ref": len(ref_index), "n_got": len(got_index), "n_common": len(common),
        "agreement": len(common) / denom if denom else 1.0,  # two empty sets agree
        "pos_max": 0.0, "pos_p99": 0.0, "ori_max": 0.0, "ori_p99": 0.0, "str_rel_max": 0.0,
    }
    if len(common):
        r = np.asarray(ref_edges, np.float64)[ia]
        g = np.asarray(got_edges, np.float64)[ib]
        pe = np.hypot(r[:, 0] - g[:, 0], r[:, 1] - g[:, 1])
        oe = wrap_angle(r[:, 2] - g[:, 2])
        oe = np.where(np.isnan(r[:, 2]) & np.isnan(g[:, 2]), 0.0, oe)
        se = np.abs(r[:, 3] - g[:, 3]) / np.maximum(np.abs(r[:, 3]), 1e-30)
        out.update(pos_max=float(pe.max()), pos_p99=float(np.quantile(pe, 0.99)),
                   ori_max=float(np.nanmax(oe)), ori_p99=float(np.nanquantile(oe, 0.99)),
                   str_rel_max=float(se.max()))
    return out
