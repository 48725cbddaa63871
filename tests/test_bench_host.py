"""Host-side pieces of bench.py: the count of tiles whose exponent takes the expanded form (it sets
the FP32 work per pair in the reported roofline), checked against a direct restatement of the
kernel's per-tile test."""
import importlib.util
import math

import numpy as np

from conftest import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("bench_host", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_expanded_fraction_matches_tile_test(sty):
    b = _bench()
    # a wide image: as at 1920 px, the smooth per-pixel offset barely moves across a 32-px tile and
    # every tile takes the expanded form (on narrow images the offset spreads tiles past the bound)
    W, H, S, D = 1920, 256, 4, 1
    planes, valid = sty.synth.records(W, H, S, D, seed=5)
    assert b.expanded_fraction(planes, valid, W, H, S, D, 0.5) == 1.0
    assert b.expanded_fraction(*sty.synth.records(70, 30, S, 1, seed=5), 70, 30, S, 1, 0.5) == 0.0
    planes = planes.copy()
    rng = np.random.default_rng(1)
    far = rng.random(planes.shape[1]) < 0.0005
    planes[0, far] += 40.0  # scattered far records push some tiles to the direct form
    got = b.expanded_fraction(planes, valid, W, H, S, D, 0.5)
    # restatement: per depth and 32 x 16 tile, mean of the valid scaled positions, max distance^2
    pscale = math.sqrt(1.4426950408889634 / (2 * 0.25))
    n = W * H * S
    exp_tiles = tiles = 0
    for d in range(D):
        for ty in range(0, H, 16):
            for tx in range(0, W, 32):
                ys, xs, ss = np.meshgrid(np.arange(ty, min(ty + 16, H)), np.arange(tx, min(tx + 32, W)),
                                         np.arange(S), indexing="ij")
                idx = (((ys * W + xs) * S + ss) + d * n).reshape(-1)
                idx = idx[valid[idx] != 0]
                if idx.size == 0:
                    continue
                p = planes[0:3, idx].astype(np.float64) * pscale
                c = p.mean(axis=1, keepdims=True)
                tiles += 1
                exp_tiles += int(((p - c) ** 2).sum(0).max() <= 16.0)
    assert tiles > 0 and 0 < exp_tiles < tiles
    assert got == exp_tiles / tiles
