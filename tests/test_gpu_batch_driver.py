"""The batch command-line driver (third-order-edge-detector_gb300/toed_batch),
the replacement of the reference's run_gpu_batch.sh: a folder of PGM images
in, <basename>_edges_gpu.txt per image out, in the reference's GPU file
format.  Each written file must equal, byte for byte, the file the library
writes for the same image detected from device memory; unreadable files are
reported and skipped."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _write_pgm(path, img, plain=False, maxval=255):
    H, W = img.shape
    with open(path, "wb") as f:
        if plain:
            f.write(f"P2\n# plain\n{W} {H}\n{maxval}\n".encode())
            f.write("\n".join(" ".join(str(int(v)) for v in row) for row in img).encode() + b"\n")
        elif maxval > 255:
            f.write(f"P5\n{W} {H}\n{maxval}\n".encode())
            f.write(img.astype(">u2").tobytes())
        else:
            f.write(f"P5\n{W} {H}\n# comment\n{maxval}\n".encode())
            f.write(img.astype(np.uint8).tobytes())


def test_batch_driver_folder(toed, oracle, synth, tmp_path):
    import torch
    toed.build()
    exe = os.path.join(os.path.dirname(toed.LIB_PATH), "toed_batch")
    assert os.path.exists(exe)
    src, out = tmp_path / "in", tmp_path / "out"
    src.mkdir()
    imgs = {}
    for k, (H, W) in enumerate([(96, 128), (200, 150), (64, 80)]):
        imgs[f"img{k}"] = synth.shapes_image(H, W, seed=2100 + k, n_shapes=4, radius_range=(10, 40),
                                             scale_to_base=False).image
    _write_pgm(src / "img0.pgm", imgs["img0"])
    _write_pgm(src / "img1.PGM", imgs["img1"])
    _write_pgm(src / "img2.pgm", imgs["img2"], plain=True)
    deep = synth.shapes_image(90, 110, seed=2110, n_shapes=4, radius_range=(10, 40),
                              scale_to_base=False).image.astype(np.int64) * 4  # 10-bit samples
    _write_pgm(src / "deep.pgm", deep, maxval=1020)
    imgs["deep"] = ((deep * 255 + 510) // 1020).astype(np.uint8)  # the driver's scaling to 0..255
    (src / "notes.txt").write_text("not an image")
    (src / "broken.pgm").write_bytes(b"P5\n64 64\n255\n" + bytes(100))
    r = subprocess.run([exe, str(src), str(out), "-s", "1.5"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 1, r.stdout + r.stderr  # one unreadable image
    assert "broken" in r.stderr and "4 edge lists written" in r.stdout
    det = toed.Detector(0)
    for name, img in imgs.items():
        got = (out / f"{name}_edges_gpu.txt").read_bytes()
        d = det.detect(torch.as_tensor(img).cuda(), sigma=1.5, out_dtype=toed.TOED_F64)
        want_path = tmp_path / f"{name}_want.txt"
        toed.write_edgels_txt(str(want_path), d["edgels"].cpu().numpy(), 10)
        assert got == want_path.read_bytes(), name
        assert d["count"] > 20
        ref = oracle.detect(img.astype(np.float64), 1.5)
        assert abs(len(ref["index"]) - d["count"]) <= max(1, d["count"] // 1000), name
    assert not (out / "notes_edges_gpu.txt").exists()
