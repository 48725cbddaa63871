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


REF_FIELDS = ("p", "wo", "ns", "ng", "le", "dir_wi", "dir_l", "ind_wi")  # float3 fields
REF_SCALARS = ("mis", "dir_pdf", "ind_mis")


def _hemisphere(n_dir: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """Cosine-ish random unit directions in the hemisphere around unit vectors n_dir."""
    v = rng.normal(size=n_dir.shape)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v = np.where((v * n_dir).sum(1, keepdims=True) < 0, -v, v)
    v = v + 0.3 * n_dir
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def ref_vertices(n: int, seed: int = 0, *, p_active: float = 0.9, n_materials: int = 3, p_flags: float = 0.1,
                 p_direct: float = 0.7, p_indirect: float = 0.8, p_emit: float = 0.05):
    """Synthetic path vertices of one depth for the reference-mode filter: points on 4 planes of a
    unit room ([-1,1]^3), shading normal = geometric normal tilted slightly, outgoing and NEE /
    continuation directions in the upper hemisphere, 'n_materials' material ids, a few emitters
    and a few vertices with non-zero stylization flags. Returns a dict of numpy arrays
    (float3 fields as [3, n] float32)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    plane = rng.integers(0, 4, n)
    axes = np.array([1, 1, 0, 2])
    sides = np.array([-1.0, 1.0, -1.0, 1.0])
    p = rng.uniform(-1.0, 1.0, size=(n, 3))
    p[np.arange(n), axes[plane]] = sides[plane]
    ng = np.zeros((n, 3))
    ng[np.arange(n), axes[plane]] = -sides[plane]  # pointing into the room
    ns = ng + 0.05 * rng.normal(size=(n, 3))
    ns /= np.linalg.norm(ns, axis=1, keepdims=True)
    wo = _hemisphere(ng, rng)
    dir_wi = _hemisphere(ng, rng)
    ind_wi = _hemisphere(ng, rng)
    has_dir = rng.random(n) < p_direct
    has_ind = rng.random(n) < p_indirect
    out = {
        "active": (rng.random(n) < p_active).astype(np.int32),
        "p": p.T.astype(np.float32), "wo": wo.T.astype(np.float32),
        "ns": ns.T.astype(np.float32), "ng": ng.T.astype(np.float32),
        "le": (np.where(rng.random((n, 1)) < p_emit, 5.0, 0.0) * rng.random((n, 3))).T.astype(np.float32),
        "mis": np.where(rng.random(n) < 0.3, rng.uniform(0.2, 1.0, n), 1.0).astype(np.float32),
        "dir_wi": (dir_wi * has_dir[:, None]).T.astype(np.float32),
        "dir_l": rng.lognormal(-1.0, 1.0, size=(3, n)).astype(np.float32),
        "dir_pdf": np.where(has_dir, rng.uniform(0.1, 3.0, n), 0.0).astype(np.float32),
        "ind_wi": (ind_wi * has_ind[:, None]).T.astype(np.float32),
        "ind_mis": np.where(rng.random(n) < 0.2, rng.uniform(0.1, 1.0, n), 1.0).astype(np.float32),
        "flags": np.where(rng.random(n) < p_flags, rng.integers(0, 16, n), 0).astype(np.uint32),
        "material": rng.integers(0, n_materials, n).astype(np.uint32),
        "in_next": rng.lognormal(-1.5, 1.0, size=(3, n)).astype(np.float32),
    }
    return {k: np.ascontiguousarray(v) for k, v in out.items()}
