"""Generate tests/golden/golden.json: known-answer vectors for the integer and style arithmetic.

The reference ships no golden vectors for this path (no tests of NL-PF, the style nodes or the
sampler). The vectors here come from two independent sources:
  * PCG32: the published output of the PCG reference demo (pcg32_srandom_r(42, 54), first six
    draws 0xa15c02b7 ... 0xcbed606e, from the pcg-c-basic distribution). The reference's
    Pcg32::new_seq_offset(seq, seed) (crates/akari_render/src/sampler/mod.rs:94-100) is exactly
    pcg32_srandom_r(seed, seq), so those six numbers pin it. Further streams are produced by the
    pure-Python restatement below, which reproduces the published six.
  * hash-grid cells and style nodes: a pure-Python (math module, FP64) restatement of the cited
    reference lines, independent of the C++ oracle.
Run: python tests/golden/make_golden.py   (deterministic; rewrites golden.json)
"""
from __future__ import annotations

import json
import math
import pathlib
import struct

HERE = pathlib.Path(__file__).resolve().parent
M64 = (1 << 64) - 1

PCG_PUBLISHED = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]


def pcg_stream(seq: int, seed: int, draws: int):
    """sampler/mod.rs:82-123: set_seq_offset then gen_u32 draws."""
    st = [0, ((seq << 1) | 1) & M64]

    def nxt():
        old = st[0]
        st[0] = (old * 0x5851F42D4C957F2D + st[1]) & M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF

    nxt()
    st[0] = (st[0] + seed) & M64
    nxt()
    return [nxt() for _ in range(draws)], list(st)


def f32(x: float) -> float:
    return struct.unpack("f", struct.pack("f", x))[0]


def hash_cell(p, pmin, pmax, res, table):
    """lm_path_filtering.rs:20-59 in float32 steps (each op rounded to f32)."""
    c = []
    for a in range(3):
        v = f32(f32(p[a] - pmin[a]) / f32(pmax[a] - pmin[a]))
        v = min(max(v, 0.0), 1.0)
        v = f32(v * float(res[a]))
        c.append(min(int(v), res[a] - 1))
    h = ((c[0] * 73856093) ^ (c[1] * 19349663) ^ (c[2] * 83492791)) & M64
    return c, h % table


# ---- style nodes (crates/akari_render/src/svm/surface/mod.rs), FP64 ------------------------
def lum709(c):
    return c[0] * 0.2126 + c[1] * 0.7152 + c[2] * 0.0722


def l2s(v):
    return v * 12.92 if v <= 0.0031308 else v ** (1 / 2.4) * 1.055 - 0.055


def s2l(v):
    return v / 12.92 if v <= 0.04045 else ((v + 0.055) / 1.055) ** 2.4


def toon(li, w):  # mod.rs:573-610
    c = [min(max(x, 0.0), 1e5) for x in li]
    lum = lum709(c)
    if lum <= 0:
        return c
    hue = [x / lum for x in c]
    if lum > 1:
        nl = math.floor(lum / w) * w
    else:
        nl = s2l(math.floor(l2s(lum) / w) * w)
    return [h * nl for h in hue]


def palette(li, depth, colors, indirect_scale, gamma):  # mod.rs:697-735
    c = list(li)
    lum = sum(c) / 3
    if depth != 0:
        c = [x / indirect_scale for x in c]
    c = [min(max(x, 0.0), 1.0) ** gamma for x in c]
    best, md = [0.0, 0.0, 0.0], 1e16
    for q in colors:
        d = sum((q[k] - c[k]) ** 2 for k in range(3))
        if d < md:
            md, best = d, list(q)
    c = [x ** (1 / gamma) for x in best]
    if depth != 0:
        nl = sum(c) / 3
        if nl != 0:
            c = [x * lum / nl for x in c]
    return c


def sat_rex(li, blend):  # mod.rs:1060-1089
    lum = sum(li) / 3
    if lum <= 0 or min(li) < 0:
        return list(li)
    cmin, cmax = min(li), max(li)
    im = [(x - cmin) / cmax for x in li]
    u = sum(im) / 3
    if u != 0:
        return [blend * lum + (1 - blend) * x * lum / u for x in im]
    return [blend * lum + (1 - blend) * lum] * 3


def toon_steps(li, t, levels):
    c = [min(max(x, 0.0), 1e5) for x in li]
    lum = lum709(c)
    if lum <= 0:
        return c
    k = sum(1 for x in t if x <= lum)
    return [x / lum * levels[k] for x in c]


def ramp_smooth(li, s, t, colors):
    c = [min(max(x, 0.0), 1e5) for x in li]
    lum = lum709(c)
    o, prev = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    for tk, ck in zip(t, colors):
        sg = 1.0 / (1.0 + math.exp(-s * (lum - tk)))
        o = [o[i] + sg * (ck[i] - prev[i]) for i in range(3)]
        prev = ck
    return o


def main():
    g = {}
    pub, _ = pcg_stream(54, 42, 6)
    assert pub == PCG_PUBLISHED, "restatement does not reproduce the published PCG32 vector"
    streams = []
    for seq, seed in [(54, 42), (0, 0), (1, 0x853C49E6748FEA9B), (123456789, 0xDEADBEEFCAFEBABE), (2**40 + 3, 7)]:
        out, st = pcg_stream(seq, seed, 8)
        streams.append({"seq": seq, "seed": seed, "draws": out, "state": st})
    g["pcg32"] = {"published_seq54_seed42": PCG_PUBLISHED, "streams": streams}

    pmin, pmax, res, table = [-1.0, -2.0, 0.5], [3.0, 2.0, 4.5], [37, 19, 23], 1 << 26
    pts = [[-1.0, -2.0, 0.5], [3.0, 2.0, 4.5], [0.0, 0.0, 1.0], [2.99, 1.99, 4.49], [-5.0, 7.0, 2.2],
           [0.123, -1.777, 3.141], [1.5, 0.25, 0.75], [2.7182817, -0.5772157, 1.4142135]]
    cells = [hash_cell(p, pmin, pmax, res, table) for p in pts]
    g["hash"] = {"pmin": pmin, "pmax": pmax, "res": res, "table": table, "points": pts,
                 "cells": [c for c, _ in cells], "index": [i for _, i in cells]}

    # style parameters are stored as float32 in sty_style_node.p: round them the same way
    F = lambda v: [f32(x) for x in v]  # noqa: E731
    inputs = [[0.0, 0.0, 0.0], [0.05, 0.02, 0.01], [0.3, 0.5, 0.2], [0.9, 0.8, 0.95], [2.5, 1.7, 3.3],
              [0.013, 0.4, 0.07], [12.0, 0.1, 5.5], [0.6, 0.6, 0.6]]
    pal = [[0.1, 0.1, 0.1], [0.8, 0.2, 0.1], [0.2, 0.7, 0.3], [0.9, 0.9, 0.8], [0.3, 0.3, 0.9]]
    palf = [F(c) for c in pal]
    g["style"] = {
        "inputs": inputs,
        "toon_w0.2": [toon(x, f32(0.2)) for x in inputs],
        "palette_d0": [palette(x, 0, palf, 1.0, 0.5) for x in inputs],
        "palette_d2": [palette(x, 2, palf, 2.0, 0.5) for x in inputs],
        "palette_colors": pal,
        "sat_rex_0.3": [sat_rex(x, f32(0.3)) for x in inputs],
        "toon_steps": [toon_steps(x, F([0.1, 0.3, 0.6]), F([0.05, 0.2, 0.45, 1.0])) for x in inputs],
        "ramp_smooth": [ramp_smooth(x, 50.0, F([0.1, 0.3, 0.6]), [F([0.1, 0.05, 0.2]), F([0.5, 0.4, 0.3]), F([1.0, 0.95, 0.8])])
                        for x in inputs],
    }
    (HERE / "golden.json").write_text(json.dumps(g, indent=1))


if __name__ == "__main__":
    main()
