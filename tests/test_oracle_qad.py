"""The MATLAB "quick and dirty" orientation mode in the oracle
(third_order_edge_detector.m:91-141): the nine derivatives cubic-interpolated
at the subpixel point.  MATLAB is not available here, so the mode is pinned
by an independent numpy restatement of the same steps (the oracle's own
derivative planes and NMS positions, Keys a = -1/2 weights, the TO vector of
cpu_toed.cpp:227-232), plus the property the mode exists for: on a disc its
orientations are closer to the true tangent than the grid-point ones."""
import numpy as np
import pytest


def _keys(t):
    a, x = -0.5, abs(t)
    if x <= 1:
        return ((a + 2) * x - (a + 3)) * x * x + 1
    if x < 2:
        return ((a * x - 5 * a) * x + 8 * a) * x - 4 * a
    return 0.0


def _qad_numpy(d9, px, py):
    x0, y0 = int(np.floor(px)), int(np.floor(py))
    wx = [_keys(px - x0 + 1 - s) for s in range(4)]
    wy = [_keys(py - y0 + 1 - s) for s in range(4)]
    blk = d9[:, y0 - 1:y0 + 3, x0 - 1:x0 + 3]
    fx, fy, fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy = np.einsum("p,kpq,q->k", np.array(wy), blk, np.array(wx))
    tix = fx * (2 * fxx * fxx + 2 * fxy * fxy) + fy * (2 * fxx * fxy + 2 * fyy * fxy) + 2 * fx * fy * fxxy + \
        fy * fy * fxyy + fx * fx * fxxx
    tiy = fx * (2 * fxx * fxy + 2 * fyy * fxy) + fy * (2 * fyy * fyy + 2 * fxy * fxy) + 2 * fx * fy * fxyy + \
        fx * fx * fxxy + fy * fy * fyyy
    return np.arctan2(tix, -tiy)


@pytest.mark.parametrize("sigma", [1.0, 1.5, 2.0])
def test_qad_oracle_matches_numpy_restatement(oracle, synth, sigma):
    img = synth.shapes_image(48, 56, seed=int(10 * sigma), n_shapes=3, radius_range=(6, 20),
                             scale_to_base=False, dtype=np.float32).image.astype(np.float64)
    g = oracle.detect(img, sigma, planes=True)
    q = oracle.detect(img, sigma, orientation="qad")
    assert len(q["index"]) > 20
    # same edgels, positions and strengths as the grid mode; only the angle differs
    assert np.array_equal(g["index"], q["index"])
    assert np.array_equal(g["edges"][:, [0, 1, 3]], q["edges"][:, [0, 1, 3]])
    d9 = oracle.planes9(img, sigma)
    pm = g["posmaps"]
    want = np.array([_qad_numpy(d9, pm[0].flat[o], pm[1].flat[o]) for o in g["index"]])
    diff = np.abs(np.angle(np.exp(1j * (want - q["edges"][:, 2]))))
    assert diff.max() < 1e-12
    assert np.abs(np.angle(np.exp(1j * (g["edges"][:, 2] - q["edges"][:, 2])))).max() > 1e-6


def test_qad_closer_to_true_tangent_on_a_disc(oracle):
    from scipy.ndimage import gaussian_filter
    H = W = 96
    cy, cx, R0, ss = 47.3, 48.6, 25.7, 8
    ys, xs = np.mgrid[0:H * ss, 0:W * ss]
    disc = (((xs + 0.5) / ss - 0.5 - cx) ** 2 + ((ys + 0.5) / ss - 0.5 - cy) ** 2) < R0 ** 2
    img = gaussian_filter(50 + 100 * disc.reshape(H, ss, W, ss).mean(axis=(1, 3)), 1.0)
    for sigma in (1.0, 2.0):
        p90 = {}
        for mode in ("grid", "qad"):
            e = oracle.detect(img, sigma, orientation=mode)["edges"]
            X, Y = e[:, 0] + 0.5, e[:, 1] + 0.5  # x_out = true position - 1/2 (cpu_toed.cpp:516)
            near = np.abs(np.hypot(X - cx, Y - cy) - R0) < 1.0
            tangent = np.arctan2(Y - cy, X - cx) + np.pi / 2
            err = np.abs(np.angle(np.exp(2j * (e[:, 2] - tangent)))) / 2  # modulo pi
            assert near.sum() > 300
            p90[mode] = np.quantile(err[near], 0.9)
        assert p90["qad"] < 0.9 * p90["grid"], p90
