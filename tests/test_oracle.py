"""The oracle is pinned before it is trusted: golden vectors (published PCG32 output and
independent FP64 restatements), analytic filter cases and a pure-Python loop on a tiny case."""
import math

import numpy as np
import pytest

from conftest import rel_err


def test_pcg32_published_vector(orc, golden):
    out, _ = orc.pcg32_streams(np.array([42], dtype=np.uint64), 54, 6)
    assert out[0].tolist() == golden["pcg32"]["published_seq54_seed42"]


def test_pcg32_streams(orc, golden):
    for s in golden["pcg32"]["streams"]:
        out, st = orc.pcg32_streams(np.array([s["seed"]], dtype=np.uint64), s["seq"], len(s["draws"]))
        assert out[0].tolist() == s["draws"]
        assert st[0].tolist() == s["state"]


def test_pcg32_stream_offsets(orc):
    seeds = np.arange(10, dtype=np.uint64) * 7919
    all_out, _ = orc.pcg32_streams(seeds, 100, 4)
    for i in range(10):
        one, _ = orc.pcg32_streams(seeds[i:i + 1], 100 + i, 4)
        assert (one[0] == all_out[i]).all()


def test_hash_cells(orc, golden):
    h = golden["hash"]
    cells, idx = orc.hash_cells(np.array(h["points"]), h["pmin"], h["pmax"], h["res"], h["table"])
    assert cells.tolist() == h["cells"]
    assert idx.tolist() == h["index"]


@pytest.mark.parametrize("key,maker", [
    ("toon_w0.2", lambda a: [a.toon(0.2)]),
    ("sat_rex_0.3", lambda a: [a.sat_rex(0.3)]),
    ("toon_steps", lambda a: [a.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0])]),
    ("ramp_smooth", lambda a: [a.ramp_smooth(50.0, [0.1, 0.3, 0.6],
                                             [(0.1, 0.05, 0.2), (0.5, 0.4, 0.3), (1.0, 0.95, 0.8)])]),
])
def test_style_nodes_golden(orc, sty, golden, key, maker):
    prog = sty.abi.style_program(maker(sty.abi))
    out = orc.style_apply(prog, 1, np.array(golden["style"]["inputs"]))
    assert rel_err(out, golden["style"][key], 1e-9).max() < 1e-12


@pytest.mark.parametrize("depth,key,scale", [(0, "palette_d0", 1.0), (2, "palette_d2", 2.0)])
def test_palette_golden(orc, sty, golden, depth, key, scale):
    prog = sty.abi.style_program([sty.abi.palette(golden["style"]["palette_colors"], scale, 0.5)])
    out = orc.style_apply(prog, depth, np.array(golden["style"]["inputs"]))
    assert rel_err(out, golden["style"][key], 1e-9).max() < 1e-12


def test_style_depth_mask(orc, sty):
    prog = sty.abi.style_program([sty.abi.toon(0.2, depth_mask=1 << 1)])
    x = np.array([[0.3, 0.5, 0.2]])
    assert np.allclose(orc.style_apply(prog, 0, x), x)
    assert not np.allclose(orc.style_apply(prog, 1, x), x)


def _tiny(sty, W=9, H=7, S=2, D=2, seed=3, **kw):
    planes, valid = sty.synth.records(W, H, S, D, seed=seed, **kw)
    return planes, valid, sty.pf.host_records(planes, valid, W, H, S, D)


def _python_filter(planes, valid, W, H, S, d, prm, out_next=None):
    """Pure-Python loop restatement of the screen filter (no style) for tiny cases."""
    N = W * H * S
    out = np.zeros((3, N))
    # the ABI carries the sigmas as float32
    sp, sx, sn = (float(np.float32(v)) for v in (prm.sigma_pos, prm.sigma_pixel, prm.sigma_nrm))
    for y in range(H):
        for x in range(W):
            for s in range(S):
                qi = (y * W + x) * S + s
                gq = d * N + qi
                if not valid[gq]:
                    continue
                sw = 0.0
                acc = [0.0, 0.0, 0.0]
                for yy in range(max(0, y - prm.radius), min(H, y + prm.radius + 1)):
                    for xx in range(max(0, x - prm.radius), min(W, x + prm.radius + 1)):
                        for t in range(S):
                            j = (yy * W + xx) * S + t
                            gj = d * N + j
                            if not valid[gj]:
                                continue
                            dp = sum((float(planes[k, gq]) - float(planes[k, gj])) ** 2 for k in range(3))
                            nd = sum(float(planes[3 + k, gq]) * float(planes[3 + k, gj]) for k in range(3))
                            a = -((xx - x) ** 2 + (yy - y) ** 2) / (2 * sx ** 2) \
                                - dp / (2 * sp ** 2) - (1 - nd) / sn ** 2
                            w = math.exp(a)
                            sw += w
                            for c in range(3):
                                v = float(planes[6 + c, gj])
                                if out_next is not None:
                                    v += float(planes[9 + c, gj]) * out_next[c, j]
                                acc[c] += w * v
                for c in range(3):
                    out[c, qi] = acc[c] / sw
    return out


def test_screen_filter_matches_python_loop(orc, sty):
    W, H, S, D = 9, 7, 2, 2
    planes, valid, rec = _tiny(sty, W, H, S, D)
    prm = sty.ScreenParams(radius=3, sigma_pixel=2.0, sigma_pos=0.7, sigma_nrm=0.4)
    out1, f1 = orc.pf_screen_filter_depth(rec, 1, prm.c(), None, want_filtered=True)
    ref1 = _python_filter(planes, valid, W, H, S, 1, prm)
    assert np.allclose(f1, ref1, rtol=1e-12, atol=1e-14)
    assert np.allclose(out1, ref1, rtol=1e-12, atol=1e-14)  # no style: out == filtered
    out0, _ = orc.pf_screen_filter_depth(rec, 0, prm.c(), None, out_next=out1)
    ref0 = _python_filter(planes, valid, W, H, S, 0, prm, out_next=out1)
    assert np.allclose(out0, ref0, rtol=1e-12, atol=1e-14)


def test_screen_filter_constant_radiance(orc, sty):
    """Furnace case: constant incoming radiance is reproduced exactly, whatever the weights."""
    W, H, S, D = 12, 10, 4, 1
    planes, valid, _ = _tiny(sty, W, H, S, D, seed=5)
    planes[6:9] = 0.37
    rec = sty.pf.host_records(planes, valid, W, H, S, D)
    out, _ = orc.pf_screen_filter_depth(rec, 0, sty.ScreenParams(4, 2.0, 0.5, 0.2).c(), None)
    m = valid.astype(bool)
    assert np.allclose(out[:, m], np.float32(0.37), rtol=1e-12)
    assert (out[:, ~m] == 0).all()


def test_screen_filter_radius0_single_sample_is_identity(orc, sty):
    """radius 0 and spp 1: the only neighbour is the record itself (weight 1)."""
    W, H, S, D = 6, 5, 1, 1
    planes, valid, rec = _tiny(sty, W, H, S, D, seed=9)
    out, _ = orc.pf_screen_filter_depth(rec, 0, sty.ScreenParams(0, 1.0, 0.5, 0.2).c(), None)
    m = valid.astype(bool)
    assert np.allclose(out[:, m], planes[6:9, m], rtol=1e-7)


def test_screen_filter_all_invalid(orc, sty):
    W, H, S, D = 5, 4, 2, 1
    planes, valid, _ = _tiny(sty, W, H, S, D)
    valid[:] = 0
    rec = sty.pf.host_records(planes, valid, W, H, S, D)
    out, _ = orc.pf_screen_filter_depth(rec, 0, sty.ScreenParams(2, 1.0, 0.5, 0.2).c(), None)
    assert (out == 0).all()


def test_f32_restatement_close_to_f64(orc, sty):
    W, H, S, D = 24, 16, 4, 1
    planes, valid, rec = _tiny(sty, W, H, S, D, seed=11)
    prm = sty.ScreenParams(8, 4.0, 0.5, 0.2)
    ref, _ = orc.pf_screen_filter_depth(rec, 0, prm.c(), None)
    got = orc.pf_screen_filter_depth_f32(rec, 0, prm.c(), None)
    m = valid.astype(bool)
    assert rel_err(got[:, m], ref[:, m]).max() < 1e-5


def test_f32_band_equals_full_image(orc, sty):
    """The band form of the FP32 restatement (rows y0..y1 only; the reference arm and the CPU
    baseline time it) gives those rows bit for bit as the full image does, styled and with a child
    input, and leaves the other rows zero."""
    W, H, S, D = 40, 24, 4, 3
    planes, valid, rec = _tiny(sty, W, H, S, D, seed=13)
    prm = sty.ScreenParams(6, 3.0, 0.5, 0.2).c()
    style = sty.c2_style()  # the toon node acts at depth 1
    n = W * H * S
    child = orc.pf_screen_filter_depth_f32(rec, 2, prm, None)
    full = orc.pf_screen_filter_depth_f32(rec, 1, prm, style, out_next=child)
    unstyled = orc.pf_screen_filter_depth_f32(rec, 1, prm, None, out_next=child)
    assert not np.array_equal(full, unstyled)  # the style does act on this depth
    y0, y1 = 9, 15
    band = orc.pf_screen_filter_depth_f32(rec, 1, prm, style, out_next=child, y0=y0, y1=y1)
    rows = slice(y0 * W * S, y1 * W * S)
    assert np.array_equal(band[:, rows], full[:, rows])
    assert (band[:, :y0 * W * S] == 0).all() and (band[:, y1 * W * S:] == 0).all()
    assert np.abs(full[:, rows]).max() > 0 and full.shape == (3, n)


def test_synthetic_records_distribution(sty):
    planes, valid = sty.synth.records(64, 48, 4, 2, seed=0)
    n = planes.shape[1]
    assert planes.dtype == np.float32 and valid.dtype == np.int32
    assert abs(valid.mean() - 0.9) < 0.02
    nrm = planes[3:6]
    assert np.allclose((nrm ** 2).sum(0), 1.0, atol=1e-5)
    rad = planes[6:9].astype(np.float64)
    assert abs(np.log(rad).mean() + 1.0) < 0.05 and abs(np.log(rad).std() - 1.5) < 0.05
    thr = planes[9:12]
    assert thr.min() >= 0 and thr.max() <= 1
    # deterministic
    p2, v2 = sty.synth.records(64, 48, 4, 2, seed=0)
    assert (p2 == planes).all() and (v2 == valid).all()
    assert n == 64 * 48 * 4 * 2


def test_screen_filter_records_matches_full_depth(orc, sty):
    """The sampled-record restatement (for checks at full image sizes) gives exactly the full-depth
    filter's values at the requested records, styled and with a child depth."""
    W, H, S, D = 21, 13, 4, 2
    planes, valid, rec = _tiny(sty, W, H, S, D, seed=17)
    prm = sty.ScreenParams(radius=5, sigma_pixel=3.0, sigma_pos=0.5, sigma_nrm=0.2)
    style = sty.c2_style()
    out1, f1 = orc.pf_screen_filter_depth(rec, 1, prm.c(), style, want_filtered=True)
    out0, f0 = orc.pf_screen_filter_depth(rec, 0, prm.c(), style, out_next=out1, want_filtered=True)
    rng = np.random.default_rng(3)
    idx = rng.choice(W * H * S, size=150, replace=False)
    o1, g1 = orc.pf_screen_filter_records(rec, 1, prm.c(), style, idx)
    o0, g0 = orc.pf_screen_filter_records(rec, 0, prm.c(), style, idx, out_next=out1)
    np.testing.assert_array_equal(o1, out1[:, idx])
    np.testing.assert_array_equal(g1, f1[:, idx])
    np.testing.assert_array_equal(o0, out0[:, idx])
    np.testing.assert_array_equal(g0, f0[:, idx])
