"""FP64 numpy restatement of the composite input encoding of the reference's NL-NRC network -- TEST
INFRASTRUCTURE ONLY.

The reference configures tiny-cuda-nn (crates/akari_integrator/src/nrc_pt.rs:1315-1349) with a
Composite encoding of its 20 + max_depth inputs: a multiresolution hash grid on the 3 position
dims, a one-blob encoding of the next 7 dims (normal, direction, roughness) and the identity on the
rest. tiny-cuda-nn (git submodule shiinamiyuki/tiny-cuda-nn, branch `ema`, no commit pinned) is not
available, so the encodings are restated from their published definitions:

  hash grid (Mueller, Evans, Schied, Keller 2022, "Instant Neural Graphics Primitives"): level l of
    L has scale s_l = N_min * b^l - 1 and resolution r_l = ceil(s_l) + 1; x in [0, 1]^3 maps to
    u = x * s_l + 0.5, cell c = floor(u), weights w = u - c (trilinear over the 8 corners). As in
    tiny-cuda-nn the cell arithmetic is FP32: s_l = exp2(l log2 b) N_min - 1 in FP32, r_l from that
    FP32 value, u = fma(x, s_l, 0.5) rounded once to FP32 (at the finest levels of deep grids s_l
    exceeds 2^24, so the FP32 cell differs from the exact one); the interpolation itself is FP64. A level
    whose r_l^3 entries fit its table (T_l = min(r_l^3 rounded up to a multiple of 8, 2^log2T))
    indexes densely (c.x + c.y r_l + c.z r_l^2), else by the spatial hash
    (c.x * 1 ^ c.y * 2654435761 ^ c.z * 805459861, in 32-bit arithmetic) mod T_l; dense indices
    are taken mod T_l too (the corner past the last cell). Inputs are clamped to [0, 1]. F features
    per entry.
  one-blob (Mueller, McWilliams, Rousselle, Gross, Novak 2019, "Neural Importance Sampling"): a
    Gaussian of standard deviation 1/B centred at x, discretised into B equal bins of [0, 1]: bin k
    gets the kernel's mass over [k/B, (k+1)/B].
  identity: the value itself.
Output order: hash-grid features (level-major), one-blob bins (dim-major), identity dims, zero
padding up to `out_width`.
"""
from __future__ import annotations

import math

import numpy as np

P1, P2 = 2654435761, 805459861


def level_scale(l, base_res, per_level_scale):
    """s_l as the FP32 evaluation exp2(l * log2(b)) * N_min - 1 (exact for b = 2)."""
    f = np.float32
    return float(f(f(np.exp2(f(l) * f(np.log2(f(per_level_scale))))) * f(base_res)) - f(1.0))


def level_geometry(levels, log2_table, base_res, per_level_scale):
    """Per level: (scale, resolution, table size, dense?) and the table offsets."""
    geo, offs, off = [], [], 0
    for l in range(levels):
        scale = level_scale(l, base_res, per_level_scale)
        res = int(math.ceil(scale)) + 1
        full = res ** 3
        size = min((full + 7) // 8 * 8, 1 << log2_table)
        geo.append((scale, res, size, full <= size))
        offs.append(off)
        off += size
    return geo, offs, off


def corner_index(c, res, size, dense):
    c = c.astype(np.uint64)
    if dense:
        return (c[..., 0] + c[..., 1] * np.uint64(res) + c[..., 2] * np.uint64(res * res)) % np.uint64(size)
    h = (c[..., 0] * np.uint64(1)) ^ (c[..., 1] * np.uint64(P1)) ^ (c[..., 2] * np.uint64(P2))
    return (h & np.uint64(0xFFFFFFFF)) % np.uint64(size)


def cells(x3, scale):
    """Cell corner and FP32 fractional weights of positions x3 at one level's scale."""
    x32 = np.clip(np.asarray(x3, dtype=np.float32), np.float32(0.0), np.float32(1.0))
    u = (x32.astype(np.float64) * scale + 0.5).astype(np.float32)  # exact product + 0.5, one rounding
    c0 = np.floor(u)
    return c0.astype(np.float64), (u - c0).astype(np.float64)


def grid_forward(x3, tables, levels, feats, log2_table, base_res, per_level_scale):
    """x3 [n, 3] (clamped to [0, 1]); tables [total_entries, feats] -> features [n, levels * feats]."""
    geo, offs, _ = level_geometry(levels, log2_table, base_res, per_level_scale)
    n = x3.shape[0]
    out = np.zeros((n, levels * feats))
    for l, (scale, res, size, dense) in enumerate(geo):
        c0, w = cells(x3, scale)
        for k in range(8):
            o = np.array([(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1], dtype=np.float64)
            wt = np.prod(np.where(o == 1, w, 1.0 - w), axis=1)
            idx = corner_index(c0 + o, res, size, dense).astype(np.int64) + offs[l]
            out[:, l * feats:(l + 1) * feats] += wt[:, None] * tables[idx]
    return out


def grid_backward(x3, dfeat, levels, feats, log2_table, base_res, per_level_scale, total):
    """Gradient of sum(dfeat * features) with respect to the tables."""
    geo, offs, _ = level_geometry(levels, log2_table, base_res, per_level_scale)
    g = np.zeros((total, feats))
    for l, (scale, res, size, dense) in enumerate(geo):
        c0, w = cells(x3, scale)
        for k in range(8):
            o = np.array([(k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1], dtype=np.float64)
            wt = np.prod(np.where(o == 1, w, 1.0 - w), axis=1)
            idx = corner_index(c0 + o, res, size, dense).astype(np.int64) + offs[l]
            np.add.at(g, idx, wt[:, None] * dfeat[:, l * feats:(l + 1) * feats])
    return g


def oneblob(x, bins):
    """x [n, d] -> [n, d * bins]: Gaussian (sigma = 1 / bins) mass over each bin of [0, 1]."""
    from scipy.special import erf
    sig = 1.0 / bins
    edges = np.arange(bins + 1) / bins
    cdf = 0.5 * (1.0 + erf((edges[None, None, :] - x[:, :, None]) / (sig * math.sqrt(2.0))))
    return (cdf[:, :, 1:] - cdf[:, :, :-1]).reshape(x.shape[0], -1)


def encode(x, tables, levels, feats, log2_table, base_res, per_level_scale, blob_dims, bins, out_width):
    g = grid_forward(x[:, :3], tables, levels, feats, log2_table, base_res, per_level_scale)
    b = oneblob(x[:, 3:3 + blob_dims], bins)
    ident = x[:, 3 + blob_dims:]
    e = np.concatenate([g, b, ident], axis=1)
    out = np.zeros((x.shape[0], out_width))
    out[:, :e.shape[1]] = e
    return out


def adam_step(w, m, v, g, tsteps, n_mlp, t, lr, b1=0.9, b2=0.99, eps=1e-8):
    """One optimiser step of the grid network, FP64: tiny-cuda-nn's Adam as the reference configures it
    (nrc_pt.rs:1195-1213: Adam nested in ExponentialDecay; tiny-cuda-nn is the git submodule
    shiinamiyuki/tiny-cuda-nn, branch `ema`, no commit pinned). Matrix parameters (the MLP weights,
    p < n_mlp) take the step with the global step count t; a non-matrix parameter (table entry)
    whose gradient is exactly zero is left as it is -- weight, moments and its own step count -- and
    the others advance their own count t_p, which sets their bias correction:
        m = b1 m + (1 - b1) g,  v = b2 v + (1 - b2) g^2,
        w -= lr (m / (1 - b1^t)) / (sqrt(v / (1 - b2^t)) + eps).
    Returns new (w, m, v, tsteps); tsteps covers the table entries only."""
    w, m, v, g = (np.asarray(a, dtype=np.float64).copy() for a in (w, m, v, g))
    tsteps = np.asarray(tsteps, dtype=np.int64).copy()
    tp = np.full(w.shape, float(t))
    upd = np.ones(w.shape, dtype=bool)
    upd[n_mlp:] = g[n_mlp:] != 0.0
    tsteps[upd[n_mlp:]] += 1
    tp[n_mlp:] = tsteps
    m[upd] = b1 * m[upd] + (1 - b1) * g[upd]
    v[upd] = b2 * v[upd] + (1 - b2) * g[upd] ** 2
    c1, c2 = 1 - b1 ** tp[upd], 1 - b2 ** tp[upd]
    w[upd] -= lr * (m[upd] / c1) / (np.sqrt(v[upd] / c2) + eps)
    return w, m, v, tsteps
