"""Adjoint of the fused detection (toed_backward_batch, torch.autograd) --
configuration: float32 images of ellipses, sigma learnable, threshold 2,
selection frozen after the forward.  Loss = sum over edgels of
(strength - 10)^2 + squared distance from (x + 0.5, y + 0.5) to the nearest
generating ellipse boundary (the output convention is true position - 0.5 px).

Checked against (a) the FP64 frozen-selection restatement differentiated by
torch autograd (the FP64 reference gradient) and (b) central FP64 finite
differences of that restatement on 256 random pixels and on sigma."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIGMA = 1.5
REL = 1e-4  # relative error bound of the gradients (target of the adjoint)


def _batch(synth, n=2, H=128, W=160, seed0=4000):
    out = []
    for k in range(n):
        si = synth.shapes_image(H, W, seed=seed0 + k, dtype=np.float32, ellipses_only=True, n_shapes=6,
                                radius_range=(12, 45), scale_to_base=False)
        out.append(si)
    return out


def _loss_terms(edg, shapes, synth):
    """Per-edgel loss with the nearest boundary points held fixed (the
    gradient of the squared distance is 2 (p - q))."""
    e = edg.to(torch.float64)
    p = e[:, :2].detach().cpu().numpy() + 0.5
    qx, qy, _ = synth.nearest_boundary_points(p[:, 0], p[:, 1], shapes)
    q = torch.as_tensor(np.stack([qx, qy], 1), dtype=torch.float64, device=e.device)
    return ((e[:, 3] - 10.0) ** 2).sum() + (((e[:, :2] + 0.5) - q) ** 2).sum()


def test_backward_vs_fp64_reference_and_fd(toed, oracle, synth):
    from oracle import frozen
    det = toed.Detector(0)
    batch = _batch(synth)
    imgs = torch.stack([torch.as_tensor(b.image) for b in batch]).cuda()
    sig = torch.tensor(SIGMA, requires_grad=True)
    x = imgs.clone().requires_grad_(True)
    edg, counts, idx = toed.differentiable_detect(x, sig, detector=det)
    assert int(counts.sum()) == edg.shape[0] > 100
    splits = torch.split(edg, counts.tolist())
    isplit = torch.split(idx, counts.tolist())
    L = sum(_loss_terms(e, b.shapes, synth) for e, b in zip(splits, batch))
    L.backward()
    g_gpu = x.grad.double().cpu().numpy()
    gs_gpu = float(sig.grad)

    # FP64 reference gradient: same selection, same loss, torch autograd in FP64
    r = oracle.default_radius(SIGMA)
    xr = torch.as_tensor(np.stack([b.image for b in batch]), dtype=torch.float64).requires_grad_(True)
    sr = torch.tensor(SIGMA, dtype=torch.float64, requires_grad=True)

    def ref_loss(xim, s):
        tot = 0.0
        for k, b in enumerate(batch):
            out = frozen.edgel_outputs(xim[k], s, isplit[k].cpu(), r)
            tot = tot + _loss_terms(out, b.shapes, synth)
        return tot

    Lr = ref_loss(xr, sr)
    Lr.backward()
    g_ref = xr.grad.numpy()
    gs_ref = float(sr.grad)
    rel_img = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    rel_sig = abs(gs_gpu - gs_ref) / abs(gs_ref)
    assert rel_img <= REL, rel_img
    assert rel_sig <= REL, (gs_gpu, gs_ref)

    # central finite differences (FP64, same selection) on 256 random pixels
    rng = np.random.default_rng(7)
    support = np.argwhere(np.abs(g_ref) > 1e-6 * np.abs(g_ref).max())
    pick = support[rng.choice(len(support), size=256, replace=False)]
    h = 1e-3
    fd = []
    with torch.no_grad():
        base = xr.detach().clone()
        for (k, i, j) in pick:
            xp = base.clone(); xp[k, i, j] += h
            xm = base.clone(); xm[k, i, j] -= h
            fd.append(float((ref_loss(xp, sr.detach()) - ref_loss(xm, sr.detach())) / (2 * h)))
        fd = np.array(fd)
        hs = 1e-5
        fd_sig = float((ref_loss(base, sr.detach() + hs) - ref_loss(base, sr.detach() - hs)) / (2 * hs))
    an = g_gpu[pick[:, 0], pick[:, 1], pick[:, 2]]
    rel_fd = np.linalg.norm(an - fd) / np.linalg.norm(fd)
    assert rel_fd <= REL, rel_fd
    assert abs(gs_gpu - fd_sig) / abs(fd_sig) <= REL, (gs_gpu, fd_sig)


def test_backward_matches_direct_call(toed, synth):
    det = toed.Detector(0)
    batch = _batch(synth, n=3, H=100, W=90, seed0=4100)
    imgs = [torch.as_tensor(b.image).cuda() for b in batch]
    res = det.detect_batch(imgs, sigma=SIGMA)
    g_out = [torch.randn_like(r["edgels"]) for r in res]
    g1, s1 = det.backward_batch(imgs, [r["index"] for r in res], g_out, sigma=SIGMA)
    g2, s2 = det.backward_batch(imgs, [r["index"] for r in res], g_out, sigma=SIGMA)
    for a, b in zip(g1, g2):
        torch.testing.assert_close(a, b, rtol=1e-5, atol=1e-6)  # shared-memory float atomics: order may vary
    assert abs(float(s1) - float(s2)) <= 1e-9 * max(1.0, abs(float(s1)))
    # an image with no edgels gets a zero gradient
    z = torch.full((40, 40), 128.0, device="cuda")
    gz, sz = det.backward_batch([z], [torch.zeros(0, dtype=torch.int32, device="cuda")],
                                [torch.zeros((0, 4), device="cuda")], sigma=SIGMA)
    assert float(gz[0].abs().max()) == 0.0 and float(sz) == 0.0


def test_backward_config_size_16x512(toed, oracle, synth):
    """The differentiable configuration at its full size: 16 float32 512x512
    ellipse images from the benchmark's generator (seeds 4000 + k), sigma
    1.5 learnable, threshold 2, the selection frozen.  GPU gradients (pixels
    and sigma) against the FP64 reference gradient and against central FP64
    finite differences on 256 random pixels and on sigma, relative error
    <= 1e-4.  A pixel's finite difference is taken over the edgels whose
    windows hold it (the loss is a sum over edgels; the others do not move)."""
    from oracle import frozen
    det = toed.Detector(0)
    batch = [synth.shapes_image(512, 512, seed=4000 + k, dtype=np.float32, ellipses_only=True)
             for k in range(16)]
    imgs = torch.stack([torch.as_tensor(b.image) for b in batch]).cuda()
    sig = torch.tensor(SIGMA, requires_grad=True)
    x = imgs.clone().requires_grad_(True)
    edg, counts, idx = toed.differentiable_detect(x, sig, detector=det)
    assert int(counts.sum()) == edg.shape[0] > 50_000
    splits = torch.split(edg, counts.tolist())
    isplit = [t.cpu() for t in torch.split(idx, counts.tolist())]
    L = sum(_loss_terms(e, b.shapes, synth) for e, b in zip(splits, batch))
    L.backward()
    g_gpu = x.grad.double().cpu().numpy()
    gs_gpu = float(sig.grad)

    r = oracle.default_radius(SIGMA)
    xr = torch.as_tensor(np.stack([b.image for b in batch]), dtype=torch.float64).requires_grad_(True)
    sr = torch.tensor(SIGMA, dtype=torch.float64, requires_grad=True)

    def img_loss(k, xim_k, s, sel=None):
        ix = isplit[k] if sel is None else isplit[k][sel]
        return _loss_terms(frozen.edgel_outputs(xim_k, s, ix, r), batch[k].shapes, synth)

    Lr = sum(img_loss(k, xr[k], sr) for k in range(len(batch)))
    Lr.backward()
    g_ref = xr.grad.numpy()
    gs_ref = float(sr.grad)
    rel_img = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    assert rel_img <= REL, rel_img
    assert abs(gs_gpu - gs_ref) / abs(gs_ref) <= REL, (gs_gpu, gs_ref)

    rng = np.random.default_rng(11)
    support = np.argwhere(np.abs(g_ref) > 1e-6 * np.abs(g_ref).max())
    pick = support[rng.choice(len(support), size=256, replace=False)]
    h, W2 = 1e-3, 2 * 512
    fd = []
    with torch.no_grad():
        base = xr.detach().clone()
        s0 = sr.detach()
        for (k, i, j) in pick:
            gi = isplit[k].numpy().astype(np.int64)
            near = (np.abs(gi // W2 / 2.0 - i) <= r + 3) & (np.abs(gi % W2 / 2.0 - j) <= r + 3)
            sel = torch.as_tensor(np.nonzero(near)[0])
            xp = base[k].clone(); xp[i, j] += h
            xm = base[k].clone(); xm[i, j] -= h
            fd.append(float((img_loss(k, xp, s0, sel) - img_loss(k, xm, s0, sel)) / (2 * h)))
        fd = np.array(fd)
        hs = 1e-5
        fd_sig = float((sum(img_loss(k, base[k], s0 + hs) for k in range(len(batch))) -
                        sum(img_loss(k, base[k], s0 - hs) for k in range(len(batch)))) / (2 * hs))
    an = g_gpu[pick[:, 0], pick[:, 1], pick[:, 2]]
    rel_fd = np.linalg.norm(an - fd) / np.linalg.norm(fd)
    assert rel_fd <= REL, rel_fd
    assert abs(gs_gpu - fd_sig) / abs(fd_sig) <= REL, (gs_gpu, fd_sig)
