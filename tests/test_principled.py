"""The reference's principled BSDF (STY_MAT_PRINCIPLED; svm/surface/principled.rs) against its FP64
oracle restatement (oracle.principled_*): the albedo table, evaluation and sampling on the device
(sty_principled_table, sty_bsdf_eval, sty_bsdf_sample, shading frame), energy and sampling
consistency, and the tracers with principled surfaces.

Tolerances: FP32 against FP64 of the same closure; at a roughness of 0.1 or more, 98 % of the values
within 1e-4 relative of max(|f|, 1e-3) and all within 1e-2 (near-mirror lobes -- roughness ~0, alpha
1e-4 -- amplify rounding of the half vector without bound and are checked by energy and sampling
consistency instead)."""
import numpy as np
import pytest

import oracle

MATS = {  # name: principled(...) keyword arguments
    "plastic": dict(base_color=(0.7, 0.3, 0.2), roughness=0.4),
    "diffuse_nospec": dict(base_color=(0.2, 0.6, 0.3), roughness=0.5, specular_ior_level=0.0),
    "metal": dict(base_color=(0.95, 0.64, 0.54), roughness=0.3, metallic=1.0),
    "glass": dict(base_color=(0.9, 0.95, 1.0), roughness=0.2, transmission=1.0, ior=1.45),
    "coated": dict(base_color=(0.1, 0.2, 0.6), roughness=0.6, coat_weight=0.44, coat_roughness=0.1),
    "mixed": dict(base_color=(0.5, 0.5, 0.4), roughness=0.35, metallic=0.24, transmission=0.3,
                  specular_tint=(0.9, 0.8, 0.7), coat_weight=0.2, coat_roughness=0.2, coat_tint=(0.9, 1.0, 0.9)),
}
GLASS = {  # name: glass(...) keyword arguments (STY_MAT_GLASS, glass.rs)
    "glass_node": dict(color=(0.9, 0.8, 0.95), roughness=0.25, ior=1.5),
    "glass_node_rough": dict(color=(1.0, 0.7, 0.5), roughness=0.6, ior=1.33),
}


def _mat(sty, name):
    return sty.scene.glass(**GLASS[name]) if name in GLASS else sty.scene.principled(**MATS[name])


def _dirs(rng, n, both=True):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    if not both:
        v[:, 2] = np.abs(v[:, 2])
    return v


def test_oracle_principled_diffuse_limit(sty):
    """No specular layer (specular_ior_level 0), no metal, glass or coat: exactly Lambert."""
    m = sty.scene.principled((0.3, 0.5, 0.7), roughness=0.8, specular_ior_level=0.0)
    rng = np.random.default_rng(0)
    wo, wi = _dirs(rng, 500), _dirs(rng, 500)
    f, pdf = oracle.principled_eval(m, wo, wi)
    same = wo[:, 2] * wi[:, 2] > 0
    k = np.abs(wi[:, 2]) / np.pi
    np.testing.assert_allclose(pdf, np.where(same, k, 0.0), rtol=1e-12, atol=0)
    np.testing.assert_allclose(f, np.where(same, k, 0.0)[:, None] * np.array([0.3, 0.5, 0.7]), rtol=1e-6, atol=1e-15)


def test_oracle_glass_is_the_dielectric_layer(sty):
    """glass.rs is the principled closure's dielectric layer on its own: with a white colour (where the
    principled transmission tint sqrt(base) equals the glass tint) and the specular, metal and coat
    layers off, the two oracle closures agree; at normal incidence the reflection is chosen with the
    Fresnel probability ((ior - 1) / (ior + 1))^2."""
    rng = np.random.default_rng(5)
    wo, wi = _dirs(rng, 4000), _dirs(rng, 4000)
    g = sty.scene.glass((1.0, 1.0, 1.0), ior=1.5, roughness=0.3)
    p = sty.scene.principled((1.0, 1.0, 1.0), roughness=0.3, ior=1.5, transmission=1.0, specular_tint=(0, 0, 0))
    fg, pg = oracle.principled_eval(g, wo, wi)
    fp, pp = oracle.principled_eval(p, wo, wi)
    np.testing.assert_allclose(fg, fp, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(pg, pp, rtol=1e-12, atol=1e-300)
    # a tinted glass scales both lobes by its colour (the principled closure would use sqrt for the
    # transmitted one)
    gt = sty.scene.glass((0.5, 0.25, 1.0), ior=1.5, roughness=0.3)
    ft, pt = oracle.principled_eval(gt, wo, wi)
    np.testing.assert_allclose(ft, fg * np.array([0.5, 0.25, 1.0]), rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(pt, pg, rtol=1e-12)
    n = 20000
    wo0 = np.tile([0.0, 0.0, 1.0], (n, 1))
    u = rng.random((n, 3))
    wis, _, ps = oracle.principled_sample(sty.scene.glass((1, 1, 1), ior=1.5, roughness=0.1), wo0, u)
    refl = wis[:, 2] > 0
    assert (refl == (u[:, 0] < 0.04)).mean() > 0.999
    assert (ps > 0).mean() > 0.99


def test_glass_scene_graph(sty):
    sg = sty.scenegraph
    nodes = {"c": {"type": "rgb", "value": [0.9, 0.95, 1.0], "colorspace": "srgb"},
             "i": {"type": "float", "value": 1.45}, "r": {"type": "float", "value": 0.1},
             "g": {"type": "glass", "color": {"id": "c"}, "ior": {"id": "i"}, "roughness": {"id": "r"}},
             "o": {"type": "output", "node": {"id": "g"}}}
    lm = sg.convert_material("Glass", {"shader": {"nodes": nodes, "output": "o"}})
    assert lm.kind == sty.scene.MAT_GLASS and not lm.warnings
    assert lm.params == pytest.approx(dict(roughness=0.1, ior=1.45))
    assert lm.alpha == pytest.approx(0.01)


def test_oracle_principled_table_limits():
    t = oracle.principled_table()  # [z, mu, roughness]
    assert np.isfinite(t).all() and t.min() >= 0 and t.max() <= 1.0 + 1e-9
    assert t[0, 1:].max() < 1e-3  # ior -> 1: no reflection away from grazing incidence
    # near-mirror at normal incidence: the Fresnel factor f0 = z^4 (ior_from_f0 clamps f0 at 0.99)
    z = np.clip(np.arange(16) / 15, 1e-4, 0.9999)
    np.testing.assert_allclose(t[:, 15, 0], np.minimum(z ** 4, 0.99), rtol=2e-3, atol=1e-4)
    assert (np.diff(t[:, 8, 8]) > 0).all()  # more reflective with higher ior


@pytest.mark.gpu
def test_principled_table_matches_oracle(sty, cuda):
    import ctypes as C
    g = (C.c_float * 4096)()
    sty.abi.check(sty.abi.lib().sty_principled_table(g))
    gpu = np.frombuffer(g, dtype=np.float32).reshape(16, 16, 16)
    ref = oracle.principled_table()
    # the grazing row (mu = 1e-4) and the ior -> 1 plane are ill-conditioned in FP32 (ior_from_f0 of
    # 1e-16 rounds to exactly 1): loose there, tight elsewhere
    np.testing.assert_allclose(gpu[1:, 1:], ref[1:, 1:], atol=2e-5)
    np.testing.assert_allclose(gpu[1:, 0], ref[1:, 0], atol=1e-2)
    assert np.isfinite(gpu).all() and gpu.min() >= 0 and gpu.max() <= 1


def _gpu_eval(sty, m, wo, wi):
    import torch
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    n = wo.shape[0]
    f = torch.zeros((n, 3), device="cuda")
    p = torch.zeros(n, device="cuda")
    import ctypes as C
    wo_d, wi_d = d(wo), d(wi)  # kept alive until the call returns
    sty.abi.check(sty.abi.lib().sty_bsdf_eval(C.byref(m), n, wo_d.data_ptr(), wi_d.data_ptr(), f.data_ptr(),
                                              p.data_ptr(), None))
    torch.cuda.synchronize()
    return f.cpu().numpy().astype(np.float64), p.cpu().numpy().astype(np.float64)


def _gpu_sample(sty, m, wo, u):
    import ctypes as C
    import torch
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    n = wo.shape[0]
    wi = torch.zeros((n, 3), device="cuda")
    f = torch.zeros((n, 3), device="cuda")
    p = torch.zeros(n, device="cuda")
    wo_d, u_d = d(wo), d(u)  # kept alive until the call returns
    sty.abi.check(sty.abi.lib().sty_bsdf_sample(C.byref(m), n, wo_d.data_ptr(), u_d.data_ptr(), wi.data_ptr(),
                                                f.data_ptr(), p.data_ptr(), None))
    torch.cuda.synchronize()
    return wi.cpu().numpy().astype(np.float64), f.cpu().numpy().astype(np.float64), p.cpu().numpy().astype(np.float64)


def _close(a, b, scale):
    return np.abs(a - b) <= 1e-4 * np.maximum(np.abs(b), 1e-3 * scale)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MATS) + sorted(GLASS))
def test_principled_eval_matches_oracle(sty, cuda, name):
    m = _mat(sty, name)
    rng = np.random.default_rng(1)
    wo, wi = _dirs(rng, 20000), _dirs(rng, 20000)
    wo32, wi32 = wo.astype(np.float32).astype(np.float64), wi.astype(np.float32).astype(np.float64)
    f, p = _gpu_eval(sty, m, wo32, wi32)
    rf, rp = oracle.principled_eval(m, wo32, wi32)
    assert np.isfinite(f).all() and np.isfinite(p).all()
    for a, b in ((f, rf), (p, rp)):
        scale = np.abs(b).max()
        ok = _close(a, b, scale)
        assert ok.mean() >= 0.98, (name, ok.mean())
        assert (np.abs(a - b) <= 1e-2 * np.maximum(np.abs(b), 1e-3 * scale)).all(), name


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MATS) + sorted(GLASS))
def test_principled_sample_matches_oracle(sty, cuda, name):
    m = _mat(sty, name)
    rng = np.random.default_rng(2)
    wo = _dirs(rng, 20000).astype(np.float32).astype(np.float64)
    u = rng.random((20000, 3)).astype(np.float32).astype(np.float64)
    wi, f, p = _gpu_sample(sty, m, wo, u)
    rwi, rf, rp = oracle.principled_sample(m, wo, u)
    same_dir = np.abs(wi - rwi).max(1) <= 1e-4
    assert same_dir.mean() >= 0.99, (name, same_dir.mean())  # lobe choices can flip at a boundary
    # sampled directions concentrate where narrow lobes peak, which amplifies FP32 rounding of the
    # half vector: 1e-3 relative here
    ok = (np.abs(p - rp) <= 1e-3 * np.maximum(rp, 1e-3 * rp.max())) & same_dir
    assert ok.mean() >= 0.98, (name, ok.mean())


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MATS) + sorted(GLASS) + ["mirror_metal", "clear_glass"])
def test_principled_energy_and_sampling_consistency(sty, cuda, name):
    """E[f/pdf] over the closure's own samples equals the sphere integral of f estimated with uniform
    directions (sampling and pdf agree: within 4 standard errors), and no energy is gained for wo
    above the surface. (From below the reference's layers are not energy conserving: the dielectric
    Fresnel of the specular and coat layers flips to 1 / ior while their weights read the
    front-side albedo table, and transmission scales radiance by ior^2; the oracle gives the same.)"""
    kw = dict(MATS.get(name, {}))
    if name == "mirror_metal":
        kw = dict(base_color=(0.9, 0.9, 0.9), roughness=0.02, metallic=1.0)
    if name == "clear_glass":
        kw = dict(base_color=(1, 1, 1), roughness=0.05, transmission=1.0, ior=1.5)
    m = sty.scene.glass(**GLASS[name]) if name in GLASS else sty.scene.principled(**kw)
    if name in GLASS:
        kw = dict(transmission=1.0)
    rng = np.random.default_rng(3)
    n = 1 << 20
    for mu in (0.9, 0.4, -0.7):
        wo = np.tile([np.sqrt(1 - mu * mu), 0.0, mu], (n, 1))
        _, f, p = _gpu_sample(sty, m, wo, rng.random((n, 3)))
        w = np.where(p[:, None] > 0, f / np.maximum(p, 1e-30)[:, None], 0.0)
        est, se_est = w.mean(0), w.std(0) / np.sqrt(n)
        if mu > 0:
            assert (est <= 1.0 + 4 * se_est + 1e-3).all(), (name, mu, est)
        if name in ("mirror_metal", "clear_glass"):
            continue  # a uniform-direction integral cannot resolve these lobes
        if mu < 0 and kw.get("transmission", 0.0) > 0:
            # from inside past the critical angle the macro-surface Fresnel is 1, so the
            # reference's lobe choice never samples transmission that rough microfacets still
            # produce (the same in the oracle): no consistency to check
            continue
        fu, _ = _gpu_eval(sty, m, wo, _dirs(rng, n))
        uni, se_uni = fu.mean(0) * 4 * np.pi, fu.std(0) * 4 * np.pi / np.sqrt(n)
        assert (np.abs(est - uni) <= 4 * np.sqrt(se_est ** 2 + se_uni ** 2) + 1e-3).all(), (name, mu, est, uni)


@pytest.mark.gpu
def test_principled_diffuse_limit_renders_like_lambert(sty, cuda):
    """The tracers with principled surfaces that reduce to Lambert (no specular layer) give the
    image of the same scene with STY_MAT_DIFFUSE materials (up to FP32 rounding)."""
    W = H = 24
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    pm = [m if max(m.emission) > 0 else sty.scene.principled(tuple(m.albedo), roughness=1.0, specular_ior_level=0.0)
          for m in mats]
    cfg = sty.scene.brpt_config(max_depth=4, inner_samples=(4, 2), repeats=2, seed=8)
    a, _ = sty.scene.Scene(pos, mids, mats, cam).brpt_render(cfg)
    b, _ = sty.scene.Scene(pos, mids, pm, cam).brpt_render(cfg)
    a, b = a.cpu().numpy(), b.cpu().numpy()
    np.testing.assert_allclose(b, a, rtol=1e-4, atol=1e-6)
    rc = sty.scene.render_config(max_depth=4, branch=8, radius_scale=(0.5,), reuse=(16,), seed=3)
    x, _ = sty.scene.Scene(pos, mids, mats, cam).render(rc)
    y, _ = sty.scene.Scene(pos, mids, pm, cam).render(rc)
    np.testing.assert_allclose(y.cpu().numpy(), x.cpu().numpy(), rtol=1e-4, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("glass_kind", ["principled", "glass_node"])
def test_principled_scene_two_integrators_agree(sty, cuda, glass_kind):
    """A Cornell box with a metal, a glass (a principled one or the glass node) and a coated principled
    box: the plain path tracer (BrPT with branching 1) and the NL-PF self-only render are both
    unbiased here and converge to the same image."""
    W = H = 24
    D = 6
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    mats = list(mats)
    mats[0] = sty.scene.principled((0.75, 0.75, 0.75), roughness=0.5, coat_weight=0.3)
    mats[1] = sty.scene.principled((0.95, 0.64, 0.54), roughness=0.25, metallic=1.0)
    mats[2] = (sty.scene.principled((0.9, 0.95, 1.0), roughness=0.15, transmission=1.0, ior=1.45)
               if glass_kind == "principled" else sty.scene.glass((0.8, 0.9, 1.0), ior=1.45, roughness=0.15))
    sc = sty.scene.Scene(pos, mids, mats, cam)
    a, _ = sc.brpt_render(sty.scene.brpt_config(max_depth=D, inner_samples=(1,), repeats=2048, seed=1))
    rc = sty.scene.render_config(max_depth=D, branch=64, repeats=32, radius_scale=(1e-4,), reuse=(8,), seed=2)
    b, _ = sc.render(rc)
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert abs(a.mean() - b.mean()) < 0.03 * b.mean(), (a.mean(), b.mean())
    sc.close()
