"""FP64 restatement of the detector's outputs with the selection frozen --
TEST INFRASTRUCTURE ONLY (the "FP64 reference gradient" of the adjoint).

Given images, sigma and the edgels' 2x-grid indices chosen by a forward
pass, recomputes each edgel's [x, y, orientation, strength] in torch FP64
exactly as the reference defines them (derivatives: cpu_toed.cpp:204-344;
TO orientation :227-232; sector, parabola fit and output :414-489, :516-529),
so that torch autograd gives d(outputs)/d(pixels, sigma) with the same
selection, and central finite differences can be taken on it.  The NMS
sector of each edgel is recomputed from its own FP64 Ix, Iy (x-major when
|Ix| >= |Iy|), as the adjoint kernel does.
"""
from __future__ import annotations

import math

import torch


def taps(sigma: torch.Tensor, r: int) -> torch.Tensor:
    """(8, 2r+3): G, Gx, Gxx, Gxxx then the +0.5-shifted set; differentiable in sigma."""
    k = torch.arange(2 * r + 3, dtype=torch.float64) - (r + 1)
    s = sigma.to(torch.float64)
    c = math.sqrt(2 * math.pi)
    rows = []
    for sh in (0.0, 0.5):
        x = k + sh
        e = torch.exp(-(x * x) / (2 * s * s))
        rows += [e / (c * s), -x * e / (c * s ** 3), (x * x - s * s) * e / (c * s ** 5),
                 x * (3 * s * s - x * x) * e / (c * s ** 7)]
    return torch.stack(rows)


def _derivs(pad, r, rho, kap, T, full):
    """Derivatives at 2x-grid points (rho, kap) of one zero-padded image."""
    NT = 2 * r + 3
    a, b = rho % 2, kap % 2
    i, j = rho // 2, kap // 2
    pp = torch.arange(NT)
    rows = (i[:, None] + 2 * (r + 1) - pp[None, :])  # image row i - p in padded coordinates
    cols = (j[:, None] + 2 * (r + 1) - pp[None, :])
    Wn = pad[rows[:, :, None], cols[:, None, :]]       # (N, NT, NT): [n, pp, qq] = I(i-p, j-q)
    trunc = ((a == 0) & (b == 0)).to(torch.float64)
    endmask = torch.ones(NT, dtype=torch.float64)
    endmask[0] = endmask[-1] = 0.0
    m = 1.0 - trunc[:, None] * (1.0 - endmask[None, :])  # zero the outer taps on sub-grid (0,0)
    X = [torch.where(b[:, None] == 1, T[4 + f][None, :], T[f][None, :]) * m for f in range(4)]
    Y = [torch.where(a[:, None] == 1, T[4 + f][None, :], T[f][None, :]) * m for f in range(4)]

    def f2(xf, yf):
        return torch.einsum("npq,nq,np->n", Wn, X[xf], Y[yf])

    out = [f2(1, 0), f2(0, 1)]  # fx = (Gx, G), fy = (G, Gy)
    if full:
        out += [f2(2, 0), f2(1, 1), f2(0, 2), f2(2, 1), f2(1, 2), f2(3, 0), f2(0, 3)]
    return out


def edgel_outputs(image: torch.Tensor, sigma: torch.Tensor, index: torch.Tensor, r: int) -> torch.Tensor:
    """(N, 4) [x, y, orientation, strength] in FP64 for the given 2x-grid
    indices of one image (H, W), differentiable in image and sigma."""
    H, W = image.shape
    W2 = 2 * W
    idx = index.to(torch.int64).cpu()
    rho, kap = idx // W2, idx % W2
    T = taps(sigma, r)
    pad = torch.nn.functional.pad(image.to(torch.float64), (r + 1, r + 1, r + 1, r + 1))
    fx, fy, fxx, fxy, fyy, fxxy, fxyy, fxxx, fyyy = _derivs(pad, r, rho, kap, T, True)
    with torch.no_grad():
        xmaj = fx.abs() >= fy.abs()
        sx = torch.where(fx >= 0, 1, -1)
        sy = torch.where(fy >= 0, 1, -1)
        ar = torch.where(xmaj, 0, sy)
        ac = torch.where(xmaj, sx, 0)
    nb = []
    for dr, dc in ((ar, ac), (sy, sx), (-ar, -ac), (-sy, -sx)):
        gx, gy = _derivs(pad, r, rho + dr, kap + dc, T, False)
        nb.append(torch.sqrt(gx * gx + gy * gy))
    MAp, MDp, MAm, MDm = nb
    m = torch.sqrt(fx * fx + fy * fy)
    nx, ny = fx / m, fy / m
    c = (sx * sy).to(torch.float64)
    t = torch.where(xmaj, c * fy / fx, c * fx / fy)
    fp = MAp * (1 - t) + MDp * t
    fm = MAm * (1 - t) + MDm * t
    s = torch.sqrt(1 + t * t)
    A = (fm + fp - 2 * m) / (2 * s * s)
    B = (fp - fm) / (2 * s)
    sst = -B / (2 * A)
    maxf = A * sst * sst + B * sst + m
    x = (kap.to(torch.float64) + sst * nx - 1) / 2
    y = (rho.to(torch.float64) + sst * ny - 1) / 2
    strength = torch.sqrt((maxf * nx) ** 2 + (maxf * ny) ** 2)
    TIx = fx * (2 * fxx * fxx + 2 * fxy * fxy) + fy * (2 * fxx * fxy + 2 * fyy * fxy) + 2 * fx * fy * fxxy + \
        fy * fy * fxyy + fx * fx * fxxx
    TIy = fx * (2 * fxx * fxy + 2 * fyy * fxy) + fy * (2 * fyy * fyy + 2 * fxy * fxy) + 2 * fx * fy * fxyy + \
        fx * fx * fxxy + fy * fy * fyyy
    ori = torch.atan2(TIx, -TIy)
    return torch.stack([x, y, ori, strength], dim=1)
