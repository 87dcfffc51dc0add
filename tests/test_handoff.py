"""After-detection outputs of the reference's drivers: the edgel text files
(written on the host, checked here without a GPU) and the column-major
curvelet hand-off (GPU)."""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden


def test_text_writer_matches_reference_cpu_file(toed, oracle):
    """toed_write_edgels_txt at 6 digits reproduces the reference's own
    data_final_output_cpu.txt byte for byte (the reference compiled where it
    lies writes it during non_maximum_suppresion, cpu_toed.cpp:541)."""
    if not oracle.ref_available():
        pytest.skip("reference build (oracle/_ref) not available")
    import ctypes
    img = golden("toed_shapes_37x53")["image"].astype(np.uint8)
    H, W = img.shape
    cap = 4 * H * W
    edges = np.zeros((cap, 4), np.float64)
    t = np.zeros(2)
    dp = ctypes.POINTER(ctypes.c_double)
    with tempfile.TemporaryDirectory() as d:
        n = oracle.ref_lib().ref_toed_detect_u8(img.ctypes.data, H, W, 1, d.encode(),
                                                edges.ctypes.data_as(dp), cap, None, None, t.ctypes.data_as(dp))
        assert n > 10
        ref_txt = open(os.path.join(d, "data_final_output_cpu.txt"), "rb").read()
        ours = os.path.join(d, "ours.txt")
        toed.write_edgels_txt(ours, edges[:n], precision=6)
        assert open(ours, "rb").read() == ref_txt


def test_text_writer_gpu_format(toed, tmp_path):
    """10 significant digits, a tab after every value, one edgel per line
    (gpu_toed.hpp:452-478); float32 lists are widened to double first."""
    e = np.array([[31.5, 12.25, -1.5707963267948966, 20.123456789012],
                  [0.0, 1e-7, np.nan, 123456.7890123]], np.float64)
    p = tmp_path / "g.txt"
    toed.write_edgels_txt(str(p), e, precision=10)
    want = "".join("".join("%.10g\t" % v for v in row) + "\n" for row in e)
    assert p.read_text() == want
    p32 = tmp_path / "f.txt"
    toed.write_edgels_txt(str(p32), e.astype(np.float32), precision=6)
    want32 = "".join("".join("%.6g\t" % float(np.float32(v)) for v in row) + "\n" for row in e)
    assert p32.read_text() == want32


@pytest.mark.gpu
@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_curvelet_columns(toed, synth, dt):
    import torch
    img = torch.as_tensor(synth.shapes_image(120, 160, seed=5, n_shapes=6, radius_range=(10, 40),
                                             scale_to_base=False, dtype=np.float32).image).cuda()
    out_dtype = toed.TOED_F64 if dt == "float64" else toed.TOED_F32
    r = toed.detect(img, sigma=1.5, out_dtype=out_dtype)
    e = r["edgels"].contiguous()
    assert e.shape[0] > 50
    cm = toed.edgels_to_columns(e)
    torch.cuda.synchronize()
    ref = e.double().t().contiguous()  # column j of the list = row j of the (4, n) array
    assert cm.shape == (4, e.shape[0]) and torch.equal(cm, ref)
    # the flat buffer is the reference's column-major layout: element (i, j) at j * n + i
    flat = cm.reshape(-1).cpu().numpy()
    n = e.shape[0]
    en = e.double().cpu().numpy()
    assert all(flat[j * n + i] == en[i, j] for i in (0, n // 2, n - 1) for j in range(4))
