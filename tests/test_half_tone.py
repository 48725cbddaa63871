"""The half-tone style node (sty_half_tone; HalfToneSurface::apply_stylization,
svm/surface/mod.rs:1180-1232): a world-space dot screen that needs the shaded point.

CPU: the FP64 oracle against a numpy restatement of the reference's steps, the node builder and the
scene-graph mapping (TRS -> affine, max_depth -> depth mask, the near-identity rule of
AffineTransform::from_matrix). GPU: sty_style_apply_at against the oracle, and a branching path
tracer render with a half-tone material against the oracle's render."""
import ctypes as C
import json
import math

import numpy as np
import pytest

from conftest import rel_err


def _numpy_half_tone(p, depth, rgb, pos):
    """mod.rs:1190-1231 step by step; p is the node's parameter list in the ABI layout."""
    ind, rs, rad, d, maxd, blend = p[:6]
    dark, light = np.array(p[6:9]), np.array(p[9:12])
    A = np.array(p[12:24]).reshape(3, 4)
    out = rgb.copy()
    if depth > maxd:
        return out
    for i, (li, x) in enumerate(zip(rgb, pos)):
        lum = li.sum() / 3.0
        if lum == 0.0:
            continue
        r = lum / rs if depth == 0 else np.sign(lum / ind) * np.floor(abs(lum / ind) + 0.5) / rs
        r = (1.0 - min(max(r, 0.0), 1.0)) * d * 0.5 * rad
        ip = np.floor((A[:, :3] @ x + A[:, 3]) / d) * d
        best = 1e16
        for c in np.ndindex(2, 2, 2):
            best = min(best, np.linalg.norm(ip + np.array(c) * d - x))
        c = (dark if best < r else light) * li
        out[i] = li + (c - li) * blend
    return out


def _node(a, **kw):
    args = dict(radius_scale=0.8, radius=1.3, grid_distance=0.07, dark_tone=(0.1, 0.15, 0.3),
                light_tone=(1.2, 1.1, 0.9), indirect_scale=0.5, blend=0.85, max_depth=2)
    args.update(kw)
    return a.half_tone(**args)


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    rgb = np.exp(rng.normal(-1.0, 1.0, size=(n, 3)))
    rgb[:5] = 0.0
    pos = rng.uniform(-2.0, 2.0, size=(n, 3))
    return rgb, pos


AFFINE = [[0.8, -0.3, 0.1, 0.25], [0.3, 0.9, 0.0, -0.1], [0.0, 0.2, 1.1, 0.05], [0, 0, 0, 1]]


@pytest.mark.parametrize("depth", [0, 1, 2, 3])
@pytest.mark.parametrize("affine", [None, AFFINE], ids=["identity", "affine"])
def test_oracle_half_tone_matches_restatement(sty, orc, depth, affine):
    nd = _node(sty.abi, affine=affine)
    prog = sty.abi.style_program([nd])
    rgb, pos = _inputs(3000, depth)
    got = orc.style_apply_at(prog, depth, rgb, pos)
    ref = _numpy_half_tone(list(nd.p[:24]), depth, rgb, pos)
    # float32 parameters, FP64 arithmetic on both sides
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-15)
    if depth > 2:
        np.testing.assert_array_equal(got, rgb)
    else:
        assert not np.allclose(got[5:], rgb[5:])
        np.testing.assert_array_equal(got[:5], 0.0)
        # every colour takes one of the two tones; with the identity map both occur (with another
        # map the corners are placed in the mapped space but measured from the unmapped point, as
        # the reference does, and the dots may miss every point)
        ratio = got[5:] / rgb[5:]
        dark = np.array([np.allclose(r, 1 + (np.array(nd.p[6:9]) - 1) * nd.p[5], rtol=1e-5) for r in ratio])
        light = np.array([np.allclose(r, 1 + (np.array(nd.p[9:12]) - 1) * nd.p[5], rtol=1e-5) for r in ratio])
        assert (dark | light).all() and light.any()
        assert dark.any() or affine is not None


def test_oracle_half_tone_dot_centres(sty, orc):
    """At a grid corner the distance is 0: every non-black colour below full brightness takes the dark
    tone at depth 0; a colour at or above radius_scale has radius 0 and takes the light tone."""
    nd = _node(sty.abi, blend=1.0)
    prog = sty.abi.style_program([nd])
    d = nd.p[3]
    pos = np.array([[3 * d, -5 * d, 7 * d], [0.0, 0.0, 0.0]], np.float64)
    dim = np.full((2, 3), 0.2)
    bright = np.full((2, 3), 2.0)
    np.testing.assert_allclose(orc.style_apply_at(prog, 0, dim, pos), dim * np.array(nd.p[6:9]), rtol=1e-6)
    np.testing.assert_allclose(orc.style_apply_at(prog, 0, bright, pos), bright * np.array(nd.p[9:12]), rtol=1e-6)
    # without a position (sty_style_apply, the screen-space filter) the node reads p = 0: a corner
    np.testing.assert_allclose(orc.style_apply(prog, 0, dim), dim * np.array(nd.p[6:9]), rtol=1e-6)


def test_half_tone_builder(sty):
    a = sty.abi
    nd = _node(a, max_depth=2)
    assert nd.kind == a.STY_STYLE_HALF_TONE and nd.depth_mask == 0b111
    assert list(nd.p[12:24]) == [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    assert _node(a, max_depth=40).depth_mask == 0xFFFFFFFF
    # within 1e-4 of the identity -> applied as the identity (geometry.rs:216-222)
    near = np.eye(4)
    near[0, 3] = 5e-5
    assert list(_node(a, affine=near).p[12:24]) == [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    far = np.eye(4)
    far[0, 3] = 2e-4
    assert _node(a, affine=far).p[15] == pytest.approx(2e-4)
    assert list(_node(a, affine=AFFINE).p[12:24]) == pytest.approx([x for r in AFFINE[:3] for x in r])
    with pytest.raises(ValueError):
        _node(a, grid_distance=0.0)
    with pytest.raises(ValueError):
        _node(a, affine=[[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0.5, 0, 0, 1]])


def test_half_tone_scene_graph(sty):
    """A sty_half_tone node of the reference's scene format maps to the node, its TRS to the affine
    map TRS::to_matrix(false) gives (scale, rotations, translation)."""
    sg, a = sty.scenegraph, sty.abi
    f = lambda v: {"type": "float", "value": v}  # noqa: E731
    rgb = lambda v: {"type": "rgb", "value": v, "colorspace": "srgb"}  # noqa: E731
    trs = {"translation": [0.1, 0.2, -0.3], "rotation": [0.3, -0.2, 0.5], "scale": [1.5, 1.0, 0.5],
           "coordinate_system": "Akari"}
    nodes = {"c": rgb([0.6, 0.6, 0.6]), "d": {"type": "diffuse", "color": {"id": "c"}},
             "h": {"type": "sty_half_tone", "surface": {"id": "d"}, "trs": trs, "radius_scale": {"id": "rs"},
                   "radius": {"id": "r"}, "indirect_scale": {"id": "is"}, "grid_distance": {"id": "g"},
                   "max_depth": 1, "blend": {"id": "b"}, "light_tone": {"id": "lt"}, "dark_tone": {"id": "dt"}},
             "rs": f(0.9), "r": f(1.1), "is": f(0.4), "g": f(0.05), "b": f(0.7),
             "lt": rgb([1.0, 0.95, 0.9]), "dt": rgb([0.05, 0.1, 0.2]),
             "o": {"type": "output", "node": {"id": "h"}}}
    lm = sg.convert_material("Dots", {"shader": {"nodes": nodes, "output": "o"}})
    ops = lm.ops[0]
    assert len(ops) == 1 and ops[0].kind == a.STY_STYLE_HALF_TONE
    nd = ops[0]
    assert list(nd.p[:6]) == pytest.approx([0.4, 0.9, 1.1, 0.05, 1.0, 0.7])
    assert nd.depth_mask == 0b11
    m = sg.trs_matrix(trs)
    assert list(nd.p[12:24]) == pytest.approx(m[:3].reshape(-1).tolist(), rel=1e-6)
    # scale first: the matrix's columns have the scale's lengths
    assert np.linalg.norm(m[:3, :3], axis=0) == pytest.approx([1.5, 1.0, 0.5])
    assert nd.p[6:9] == pytest.approx(sg.const_rgb(nodes, {"id": "dt"}))
    json.dumps(nodes)  # the fixture is plain JSON


@pytest.mark.gpu
@pytest.mark.parametrize("depth", [0, 1, 3])
@pytest.mark.parametrize("affine", [None, AFFINE], ids=["identity", "affine"])
def test_half_tone_matches_oracle(sty, orc, cuda, depth, affine):
    import torch
    prog = sty.abi.style_program([sty.abi.sat_rex(0.3), _node(sty.abi, affine=affine)])
    rgb, pos = _inputs(50000, 7 + depth)
    x = torch.from_numpy(rgb.astype(np.float32)).cuda()
    p = torch.from_numpy(pos.astype(np.float32)).cuda()
    y = torch.empty_like(x)
    sty.check(sty.lib().sty_style_apply_at(C.byref(prog), depth, x.data_ptr(), p.data_ptr(), y.data_ptr(),
                                           x.shape[0], None))
    torch.cuda.synchronize()
    got = y.cpu().numpy()
    ref = orc.style_apply_at(prog, depth, rgb.astype(np.float32).astype(np.float64),
                             pos.astype(np.float32).astype(np.float64))
    err = rel_err(got, ref, 1e-6).max(axis=1)
    # a point within float32 rounding of a dot edge or a cell boundary may take the other tone
    bad = err > 1e-5
    assert bad.sum() <= 50000 * 2e-4, f"{bad.sum()} records off (max {err.max():.3e})"
    # a null position pointer is p = 0 (sty_style_apply's behaviour)
    sty.check(sty.lib().sty_style_apply_at(C.byref(prog), depth, x.data_ptr(), None, y.data_ptr(), x.shape[0], None))
    z = torch.empty_like(x)
    sty.check(sty.lib().sty_style_apply(C.byref(prog), depth, x.data_ptr(), z.data_ptr(), x.shape[0], None))
    torch.cuda.synchronize()
    assert torch.equal(y, z)


@pytest.mark.gpu
def test_brpt_half_tone_matches_oracle(sty, orc, cuda):
    """The tracer hands the shaded point to the node at every vertex and at the light sample."""
    from test_brpt import _camv, _mats
    W, H, D = 24, 20, 4
    style = (0, -1, -1, -1)
    pos, mids, mats, cam = sty.scene.cornell_box(W, H, style=style, light_style=style)
    progs = [sty.abi.style_program([_node(sty.abi, grid_distance=0.11, max_depth=3, blend=0.9)])]
    sc = sty.scene.Scene(pos, mids, mats, cam)
    inner = (4, 3, 2)
    cfg = sty.scene.brpt_config(max_depth=D, inner_samples=inner, repeats=2, vram_mb=256, seed=23)
    film, st = sc.brpt_render(cfg, progs)
    img = film.cpu().numpy()
    ref = orc.brpt(pos, mids, _mats(sty, mats), _camv(cam), progs, D, inner, repeats=2, seed=23)
    plain = orc.brpt(pos, mids, _mats(sty, mats), _camv(cam), (), D, inner, repeats=2, seed=23)
    assert np.isfinite(img).all() and st.vertices > 0
    assert np.abs(ref - plain).max() > 0.05 * plain.mean()   # the screen changes the image
    scale = max(ref.mean(), 1e-3)
    err = np.abs(img - ref).max(2) / np.maximum(ref.max(2), scale)
    # hits within float32 rounding of a dot edge take the other tone: a few more pixels than the
    # un-screened comparison may differ
    assert np.mean(err <= 1e-3) >= 0.95, (np.mean(err > 1e-3), err.max())
    assert abs(img.mean() - ref.mean()) <= 5e-3 * ref.mean(), (img.mean(), ref.mean())
    sc.close()


def test_half_tone_radius_math():
    """radius = (1 - clamp(lum / radius_scale)) * d / 2 * radius at depth 0 (mod.rs:1201-1207)."""
    lum, rs, d, rad = 0.2, 0.8, 0.07, 1.3
    assert (1 - lum / rs) * d * 0.5 * rad == pytest.approx(0.034125)
    assert math.floor(-0.5 / 0.07) == -8


@pytest.mark.gpu
def test_ref_filter_half_tone_matches_oracle(sty, orc, cuda):
    """The reference-mode filter styles each record's filtered radiance at the record's own point."""
    from test_pf_ref import _gpu, _setup
    arr, mats, _, rng = _setup(sty, n=6000, seed=5)
    a = sty.abi
    progs = sty.pf_ref.programs([
        a.style_program([_node(a, grid_distance=0.05, max_depth=3)]),
        a.style_program([a.sat_rex(0.4), _node(a, grid_distance=0.09, max_depth=3, affine=AFFINE)]),
    ])
    prm = sty.pf_ref.RefParams(depth=1, radius=0.08, reuse=4, smis=True, cluster=False)
    st, ref_out, ref_nb, _, ref_rng = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    assert st == 0
    out, nb, _, r = _gpu(sty, arr, mats, progs, rng, prm)
    assert (nb == ref_nb).all() and (r == ref_rng).all()
    act = arr["active"].astype(bool)
    err = rel_err(out[:, act], ref_out[:, act], 1e-4).max(axis=0)
    # a record within float32 rounding of a dot edge may take the other tone
    assert np.mean(err < 1e-5) >= 0.99, (np.mean(err >= 1e-5), err.max())


@pytest.mark.gpu
def test_half_tone_rejects_zero_spacing(sty, cuda):
    import torch
    nd = _node(sty.abi)
    nd.p[3] = 0.0
    prog = sty.abi.style_program([nd])
    x = torch.ones(4, 3, device="cuda")
    with pytest.raises(sty.abi.StyError, match="invalid style program"):
        sty.check(sty.lib().sty_style_apply_at(C.byref(prog), 0, x.data_ptr(), x.data_ptr(), x.data_ptr(), 4, None))
