"""Seeded synthetic path-vertex records for the screen-space NL-PF workload.

Stands in for path-vertex dumps of a real scene (the reference's teaser geometry is not
available). Distributions, per record (pixel x, y; sample s; depth d):
  position  = U[-1, 1]^3 + o(x, y), o(x, y) = scale * (2u - 1, 2v - 1, 0.5 sin(2 pi u) cos(2 pi v)),
              u = (x + 0.5) / W, v = (y + 0.5) / H  (smooth per-pixel offset)
  normal    = von Mises-Fisher(kappa) around a per-8x8-pixel-tile mean direction
              (Wood 1994 sampler; tile means uniform on the sphere)
  radiance  = lognormal(mu, sigma) per channel
  throughput= U[0, 1]^3
  valid     = 0 with probability p_invalid, else 1
All draws come from numpy's PCG64 seeded with `seed`; each depth draws from its own
sub-stream, so depths can be generated independently.
"""
from __future__ import annotations

import numpy as np

FIELDS = ("px", "py", "pz", "nx", "ny", "nz", "rr", "rg", "rb", "tr", "tg", "tb")


def _vmf_around(mu: np.ndarray, kappa: float, rng: np.random.Generator) -> np.ndarray:
    """Wood (1994) sampler of the 3-D von Mises-Fisher distribution around unit vectors mu."""
    n = mu.shape[0]
    xi = rng.random(n)
    w = 1.0 + np.log(xi + (1.0 - xi) * np.exp(-2.0 * kappa)) / kappa
    phi = 2.0 * np.pi * rng.random(n)
    r = np.sqrt(np.clip(1.0 - w * w, 0.0, None))
    local = np.stack([r * np.cos(phi), r * np.sin(phi), w], axis=1)
    # orthonormal frame around mu
    a = np.where(np.abs(mu[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(a, mu)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(mu, t)
    v = local[:, :1] * t + local[:, 1:2] * b + local[:, 2:3] * mu
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def records(width: int, height: int, spp: int, depths: int, seed: int = 0, *,
            kappa: float = 20.0, mu: float = -1.0, sigma: float = 1.5, p_invalid: float = 0.1,
            offset_scale: float = 4.0, tile: int = 8):
    """Return (planes, valid): planes float32 [12, depths*height*width*spp] in FIELDS order,
    valid int32 [depths*height*width*spp]; record index ((d*H + y)*W + x)*spp + s."""
    n_d = width * height * spp
    planes = np.empty((12, depths * n_d), dtype=np.float32)
    valid = np.empty(depths * n_d, dtype=np.int32)
    ys, xs = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    u = ((xs + 0.5) / width).reshape(-1)
    v = ((ys + 0.5) / height).reshape(-1)
    off = offset_scale * np.stack([2 * u - 1, 2 * v - 1, 0.5 * np.sin(2 * np.pi * u) * np.cos(2 * np.pi * v)], 1)
    off = np.repeat(off, spp, axis=0)  # per record
    tiles_x = (width + tile - 1) // tile
    tiles_y = (height + tile - 1) // tile
    tile_id = np.repeat(((ys // tile) * tiles_x + (xs // tile)).reshape(-1), spp)
    ss = np.random.SeedSequence(seed)
    for d, child in enumerate(ss.spawn(depths)):
        rng = np.random.Generator(np.random.PCG64(child))
        sl = slice(d * n_d, (d + 1) * n_d)
        pos = rng.uniform(-1.0, 1.0, size=(n_d, 3)) + off
        tmu = rng.normal(size=(tiles_x * tiles_y, 3))
        tmu /= np.linalg.norm(tmu, axis=1, keepdims=True)
        nrm = _vmf_around(tmu[tile_id], kappa, rng)
        rad = rng.lognormal(mu, sigma, size=(n_d, 3))
        thr = rng.random((n_d, 3))
        val = (rng.random(n_d) >= p_invalid).astype(np.int32)
        for k in range(3):
            planes[k, sl] = pos[:, k]
            planes[3 + k, sl] = nrm[:, k]
            planes[6 + k, sl] = rad[:, k]
            planes[9 + k, sl] = thr[:, k]
        valid[sl] = val
    return planes, valid
