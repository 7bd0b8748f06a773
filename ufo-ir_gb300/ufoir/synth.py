"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark workloads (no public dataset is involved).

- Random-ellipse phantom: ``count`` ellipses with additive densities U[0, 1],
  centres, semi-axes and rotations uniform inside a disc of the phantom's
  side P, the P x P phantom centred in an n x n grid (offset (n - P) // 2).
- Random-polygon phantom: convex polygons of 3..8 vertices that overwrite
  with density U[0, 1].
- Poisson noise on line integrals p: kappa = 4 / max(p),
  N ~ Poisson(I0 exp(-kappa p)), y = -ln(max(N, 1) / I0) / kappa.
"""
from __future__ import annotations

import numpy as np


def ellipse_phantom(n: int, phantom: int, count: int = 10, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    vol = np.zeros((n, n), np.float32)
    off = (n - phantom) // 2
    r = phantom / 2.0
    yy, xx = np.mgrid[0:phantom, 0:phantom].astype(np.float64)
    xx = xx + 0.5 - r
    yy = yy + 0.5 - r
    inside = np.zeros((phantom, phantom), np.float64)
    for _ in range(count):
        rad = 0.7 * r * np.sqrt(rng.random())
        ang = 2 * np.pi * rng.random()
        cx, cy = rad * np.cos(ang), rad * np.sin(ang)
        a = r * (0.05 + 0.3 * rng.random())
        b = r * (0.05 + 0.3 * rng.random())
        phi = np.pi * rng.random()
        dens = rng.random()
        c, s = np.cos(phi), np.sin(phi)
        # evaluate inside the ellipse's bounding box only
        ext = max(a, b)
        x0 = max(0, int(np.floor(cx + r - ext)) - 1)
        x1 = min(phantom, int(np.ceil(cx + r + ext)) + 2)
        y0 = max(0, int(np.floor(cy + r - ext)) - 1)
        y1 = min(phantom, int(np.ceil(cy + r + ext)) + 2)
        if x0 >= x1 or y0 >= y1:
            continue
        bx = xx[y0:y1, x0:x1] - cx
        by = yy[y0:y1, x0:x1] - cy
        u = bx * c + by * s
        v = -bx * s + by * c
        mask = (u / a) ** 2 + (v / b) ** 2 <= 1.0
        inside[y0:y1, x0:x1][mask] += dens
    disc = xx ** 2 + yy ** 2 <= r * r
    inside[~disc] = 0.0
    vol[off:off + phantom, off:off + phantom] = inside.astype(np.float32)
    return vol


def polygon_phantom(n: int, phantom: int, count: int = 8, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    vol = np.zeros((n, n), np.float32)
    off = (n - phantom) // 2
    r = phantom / 2.0
    yy, xx = np.mgrid[0:phantom, 0:phantom].astype(np.float64)
    xx = xx + 0.5 - r
    yy = yy + 0.5 - r
    img = np.zeros((phantom, phantom), np.float64)
    for _ in range(count):
        k = int(rng.integers(3, 9))
        rad = 0.6 * r * np.sqrt(rng.random())
        ang = 2 * np.pi * rng.random()
        cx, cy = rad * np.cos(ang), rad * np.sin(ang)
        size = r * (0.1 + 0.3 * rng.random())
        th = np.sort(rng.random(k) * 2 * np.pi)
        px, py = cx + size * np.cos(th), cy + size * np.sin(th)
        inside = np.ones_like(img, bool)
        for i in range(k):
            x0, y0, x1, y1 = px[i], py[i], px[(i + 1) % k], py[(i + 1) % k]
            inside &= (x1 - x0) * (yy - y0) - (y1 - y0) * (xx - x0) >= 0
        img[inside] = rng.random()
    vol[off:off + phantom, off:off + phantom] = img.astype(np.float32)
    return vol


def poisson_noise(sino: np.ndarray, i0: float, seed: int = 0):
    """Returns (noisy sinogram, kappa)."""
    rng = np.random.default_rng(seed)
    p = np.asarray(sino, np.float64)
    mx = float(p.max())
    kappa = 4.0 / mx if mx > 0 else 1.0
    counts = rng.poisson(i0 * np.exp(-kappa * p))
    y = -np.log(np.maximum(counts, 1) / i0) / kappa
    return y.astype(np.float32), kappa


def phantom_for(n: int, phantom: int, kind: str = "ellipses", seed: int = 0) -> np.ndarray:
    if kind == "ellipses":
        return ellipse_phantom(n, phantom, 10, seed)
    if kind == "polygons":
        return polygon_phantom(n, phantom, 8, seed)
    raise ValueError(kind)
