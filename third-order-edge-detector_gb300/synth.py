"""Seeded synthetic workloads for the TOED hot path.

The reference benchmarks on no public dataset (its sample images carry no
expected outputs), so seeded synthetic images with the workload shapes stand
in for every configuration:

* ``shapes_image``  -- filled ellipses and convex polygons on a background of
  128, Gaussian blur, additive Gaussian noise (the detector workloads: one
  752x480 uint8 image; 1920x1080 / 3840x2160 float32; the uneven batch of 64
  images in [256, 2048]^2; the 16 x 512^2 differentiable batch).
* ``ridge_map``     -- cubic Bezier curves rasterised as Gaussian ridges plus
  uniform noise, clipped to [0, 1] (the subpixel TO-correction workload).

Everything is numpy with a PCG64 generator, so a seed names an input exactly.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BASE_W, BASE_H, BASE_SHAPES = 752, 480, 20


@dataclass
class Ellipse:
    cx: float
    cy: float
    a: float  # semi-axis along the rotated x axis
    b: float
    theta: float
    intensity: float


@dataclass
class Polygon:
    vertices: np.ndarray  # (k, 2) x, y in counter-clockwise angular order
    intensity: float


@dataclass
class ShapeImage:
    image: np.ndarray
    shapes: list = field(default_factory=list)


def gaussian_blur(img: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur, radius ceil(4 sigma), reflect padding, float64."""
    if sigma <= 0:
        return img.astype(np.float64)
    r = int(math.ceil(4 * sigma))
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-(x * x) / (2 * sigma * sigma))
    k /= k.sum()
    out = img.astype(np.float64)
    for axis in (0, 1):
        pad = [(0, 0), (0, 0)]
        pad[axis] = (r, r)
        p = np.pad(out, pad, mode="reflect")
        acc = np.zeros_like(out)
        n = out.shape[axis]
        for t in range(2 * r + 1):
            sl = [slice(None), slice(None)]
            sl[axis] = slice(t, t + n)
            acc += k[t] * p[tuple(sl)]
        out = acc
    return out


def _raster_ellipse(canvas, e: Ellipse):
    H, W = canvas.shape
    R = max(e.a, e.b) + 1
    x0, x1 = max(0, int(e.cx - R)), min(W, int(e.cx + R) + 2)
    y0, y1 = max(0, int(e.cy - R)), min(H, int(e.cy + R) + 2)
    if x0 >= x1 or y0 >= y1:
        return
    ys, xs = np.mgrid[y0:y1, x0:x1].astype(np.float64)
    dx, dy = xs - e.cx, ys - e.cy
    c, s = math.cos(e.theta), math.sin(e.theta)
    u = (dx * c + dy * s) / e.a
    v = (-dx * s + dy * c) / e.b
    m = (u * u + v * v) <= 1.0
    canvas[y0:y1, x0:x1][m] = e.intensity


def _raster_polygon(canvas, p: Polygon):
    H, W = canvas.shape
    vx, vy = p.vertices[:, 0], p.vertices[:, 1]
    x0, x1 = max(0, int(vx.min())), min(W, int(vx.max()) + 2)
    y0, y1 = max(0, int(vy.min())), min(H, int(vy.max()) + 2)
    if x0 >= x1 or y0 >= y1:
        return
    ys, xs = np.mgrid[y0:y1, x0:x1].astype(np.float64)
    inside = np.ones(xs.shape, bool)
    k = len(vx)
    for t in range(k):
        ax, ay = vx[t], vy[t]
        bx, by = vx[(t + 1) % k], vy[(t + 1) % k]
        # counter-clockwise vertices: inside is to the left of every edge
        inside &= ((bx - ax) * (ys - ay) - (by - ay) * (xs - ax)) >= 0
    canvas[y0:y1, x0:x1][inside] = p.intensity


def shapes_image(H: int, W: int, seed: int, n_shapes: int | None = None,
                 radius_range=(10.0, 120.0), blur_sigma: float = 1.0, noise_std: float = 3.0,
                 dtype=np.uint8, ellipses_only: bool = False, scale_to_base: bool = True) -> ShapeImage:
    """Ellipses / convex polygons on 128, blurred, noisy.

    With ``scale_to_base`` the shape count scales with the area ratio and the
    radii with the width ratio to the 752x480 base image.  uint8 output is
    rounded and clipped; float32 output is clipped to [0, 255].
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    if n_shapes is None:
        n_shapes = BASE_SHAPES
        if scale_to_base:
            n_shapes = max(1, int(round(BASE_SHAPES * (H * W) / (BASE_H * BASE_W))))
    rscale = (W / BASE_W) if scale_to_base else 1.0
    rlo, rhi = radius_range[0] * rscale, radius_range[1] * rscale
    canvas = np.full((H, W), 128.0)
    shapes = []
    for _ in range(n_shapes):
        cx, cy = rng.uniform(0, W), rng.uniform(0, H)
        inten = rng.uniform(30, 220)
        if ellipses_only or rng.uniform() < 0.5:
            e = Ellipse(cx, cy, rng.uniform(rlo, rhi), rng.uniform(rlo, rhi), rng.uniform(0, math.pi),
                        inten)
            _raster_ellipse(canvas, e)
            shapes.append(e)
        else:
            k = int(rng.integers(3, 9))
            R = rng.uniform(rlo, rhi)
            ang = np.sort(rng.uniform(0, 2 * math.pi, size=k))
            verts = np.stack([cx + R * np.cos(ang), cy + R * np.sin(ang)], axis=1)
            p = Polygon(verts, inten)
            _raster_polygon(canvas, p)
            shapes.append(p)
    img = gaussian_blur(canvas, blur_sigma)
    img = img + rng.normal(0.0, noise_std, size=img.shape)
    if np.dtype(dtype) == np.uint8:
        img = np.clip(np.rint(img), 0, 255).astype(np.uint8)
    else:
        img = np.clip(img, 0, 255).astype(dtype)
    return ShapeImage(img, shapes)


def uneven_batch(n_images: int = 64, seed0: int = 3000, lo: int = 256, hi: int = 2048,
                 sigma_noise=(1.0, 8.0), dtype=np.float32):
    """The uneven batch: sizes U[lo, hi] rounded to multiples of 4, seeds seed0+k."""
    out = []
    for k in range(n_images):
        rng = np.random.Generator(np.random.PCG64(seed0 + k))
        W = int(round(rng.uniform(lo, hi) / 4.0)) * 4
        H = int(round(rng.uniform(lo, hi) / 4.0)) * 4
        std = float(rng.uniform(*sigma_noise))
        out.append(shapes_image(H, W, seed=seed0 + k, noise_std=std, dtype=dtype).image)
    return out


def uneven_batch_shapes(n_images: int = 64, seed0: int = 3000, lo: int = 256, hi: int = 2048):
    """Sizes of ``uneven_batch`` without rasterising (for planning and tests)."""
    sizes = []
    for k in range(n_images):
        rng = np.random.Generator(np.random.PCG64(seed0 + k))
        W = int(round(rng.uniform(lo, hi) / 4.0)) * 4
        H = int(round(rng.uniform(lo, hi) / 4.0)) * 4
        sizes.append((H, W))
    return sizes


def _bezier(p0, p1, p2, p3, t):
    u = 1 - t
    return (u ** 3)[:, None] * p0 + (3 * u * u * t)[:, None] * p1 + (3 * u * t * t)[:, None] * p2 + \
        (t ** 3)[:, None] * p3


def ridge_map(H: int = 2048, W: int = 2048, seed: int = 5000, n_curves: int = 40,
              width: float = 1.5, noise=(0.0, 0.05), dtype=np.float32) -> np.ndarray:
    """Edge-probability map: cubic Bezier ridges (Gaussian cross-section of
    std ``width``, peak U[0.5, 1]) + uniform noise, clipped to [0, 1]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    E = np.zeros((H, W), np.float64)
    rad = int(math.ceil(3 * width))
    for _ in range(n_curves):
        pts = rng.uniform([0, 0], [W, H], size=(4, 2))
        peak = rng.uniform(0.5, 1.0)
        L = sum(np.linalg.norm(pts[i + 1] - pts[i]) for i in range(3))
        ns = max(8, int(L * 2))
        c = _bezier(pts[0], pts[1], pts[2], pts[3], np.linspace(0, 1, ns))
        # ridge = max over curve samples of a Gaussian bump, splatted on the
        # (2 rad + 2)^2 pixel window around each sample
        offs = np.arange(-rad, rad + 2)
        ox, oy = np.meshgrid(offs, offs)
        xs = np.floor(c[:, 0])[:, None].astype(np.int64) + ox.ravel()[None, :]
        ys = np.floor(c[:, 1])[:, None].astype(np.int64) + oy.ravel()[None, :]
        d2 = (xs - c[:, 0:1]) ** 2 + (ys - c[:, 1:2]) ** 2
        ok = (xs >= 0) & (xs < W) & (ys >= 0) & (ys < H)
        np.maximum.at(E, (ys[ok], xs[ok]), peak * np.exp(-d2[ok] / (2 * width * width)))
    E += rng.uniform(noise[0], noise[1], size=E.shape)
    return np.clip(E, 0.0, 1.0).astype(dtype)


def ellipse_closest(px, py, e: Ellipse):
    """Closest point on the boundary of ellipse ``e`` to each (px, py) and
    its distance (FP64; Newton on the parametric angle in the first
    quadrant of the ellipse frame from three starts -- radial and both axes --
    keeping the nearest)."""
    px = np.asarray(px, np.float64)
    py = np.asarray(py, np.float64)
    c, s = math.cos(e.theta), math.sin(e.theta)
    dx, dy = px - e.cx, py - e.cy
    u0 = dx * c + dy * s
    v0 = -dx * s + dy * c
    su, sv = np.where(u0 < 0, -1.0, 1.0), np.where(v0 < 0, -1.0, 1.0)
    u, v = np.abs(u0), np.abs(v0)
    a, b = e.a, e.b
    best_d = best_t = None
    for t0 in (np.arctan2(a * v, b * u), np.zeros_like(u), np.full_like(u, math.pi / 2)):
        t = t0.copy()
        for _ in range(16):
            ct, st = np.cos(t), np.sin(t)
            f = (a * a - b * b) * st * ct - u * a * st + v * b * ct
            fp = (a * a - b * b) * (ct * ct - st * st) - u * a * ct - v * b * st
            t = np.clip(t - f / np.where(np.abs(fp) < 1e-30, 1e-30, fp), 0.0, math.pi / 2)
        d = np.hypot(u - a * np.cos(t), v - b * np.sin(t))
        if best_d is None:
            best_d, best_t = d, t
        else:
            better = d < best_d
            best_d, best_t = np.where(better, d, best_d), np.where(better, t, best_t)
    qu, qv = su * a * np.cos(best_t), sv * b * np.sin(best_t)
    qx = e.cx + qu * c - qv * s
    qy = e.cy + qu * s + qv * c
    return best_d, qx, qy


def ellipse_distance(px, py, e: Ellipse) -> np.ndarray:
    """Euclidean distance from points to the boundary of ellipse ``e``."""
    return ellipse_closest(px, py, e)[0]


def nearest_boundary_points(px, py, shapes):
    """For each point, the closest boundary point over all ellipses of
    ``shapes`` (polygons are ignored): returns (qx, qy, distance)."""
    best = None
    for e in shapes:
        if not isinstance(e, Ellipse):
            continue
        d, qx, qy = ellipse_closest(px, py, e)
        if best is None:
            best = [qx, qy, d]
        else:
            m = d < best[2]
            best = [np.where(m, qx, best[0]), np.where(m, qy, best[1]), np.where(m, d, best[2])]
    return best
