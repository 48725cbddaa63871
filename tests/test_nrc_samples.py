"""NL-NRC data path: training and query rows generated by the tracer (sty_nrc_samples), and the
cache trained on them by the project's own kernels against the cache-free render it replaces.

The row layouts follow write_nrc_inputs (crates/akari_integrator/src/nrc_pt.rs:583-663) and
xyz_to_spherical_normalized (crates/akari_render/src/geometry.rs:342-346); the training targets
are the self-reuse estimator of the NL-PF render (lm_path_filtering.rs:758-972 with a one-vertex
neighbourhood), so their depth-0 sum must reproduce that render's film.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W = H = 32
D = 4


@pytest.fixture(scope="module")
def cornell(sty, cuda):
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    return sty.scene.Scene(pos, mids, mats, cam), mats


def _self_only(sty, seed, branch, repeats=1):
    return sty.scene.render_config(max_depth=D, branch=branch, repeats=repeats, radius_scale=(1e-4,), reuse=(8,),
                                   smis=False, seed=seed)


def test_train_rows_are_the_traced_vertices(sty, cornell):
    """Same seed, same paths: one training row per traced vertex, and the depth-0 targets are the
    self-reuse render's film (film = sum over a pixel's paths / spp)."""
    sc, mats = cornell
    spp, seed = 4, 21
    x, y = sc.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, spp, D, layout=sty.scene.NRC_ROWS_REF, seed=seed)
    film, nv = sc.render(_self_only(sty, seed, spp))
    assert x.shape[0] == nv > 0
    x = x.cpu().numpy()
    y = y.cpu().numpy()
    assert x.shape[1] == 20 + D
    depth = x[:, 19:].argmax(1)
    counts = np.bincount(depth, minlength=D + 1)
    assert 0 < counts[0] <= W * H * spp
    assert (np.diff(counts) <= 0).all(), counts  # a path that ends never comes back
    got = y[depth == 0].astype(np.float64).sum(0) / spp
    want = film.cpu().numpy().reshape(-1, 3).sum(0)
    np.testing.assert_allclose(got, want, rtol=1e-4)


def test_train_rows_deterministic(sty, cornell):
    """Rows are written depth-major in path order (a prefix sum, not an atomic counter), so a seed
    gives the same rows, and a cache trained on them the same parameters, on every run."""
    sc, _ = cornell
    a = sc.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, 2, D, seed=17)
    b = sc.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, 2, D, seed=17)
    assert bool((a[0] == b[0]).all()) and bool((a[1] == b[1]).all())
    params = []
    for _ in range(2):
        net = sty.nrc.NRC(sty.nrc.config(precision=sty.nrc.STY_NRC_FP32, batch_size=1 << 12, seed=3))
        net.train(a[0], a[1], n_iters=4, want_loss=False)
        params.append(net.save_params())
        net.close()
    assert (params[0] == params[1]).all()


def test_reference_row_layout(sty, cornell):
    sc, mats = cornell
    x, _ = sc.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, 2, D, layout=sty.scene.NRC_ROWS_REF, seed=3)
    x = x.cpu().numpy().astype(np.float64)
    assert np.isfinite(x).all()
    assert (x[:, :3] >= -1e-6).all() and (x[:, :3] <= 1 + 1e-6).all()
    for c0 in (3, 6):  # unit normal / direction stored as v * 0.5 + 0.5
        v = x[:, c0:c0 + 3] * 2 - 1
        np.testing.assert_allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-5)
    assert (x[:, 9] == 1.0).all()  # diffuse roughness
    alb = np.array([m.albedo[:] for m in mats], np.float32).astype(np.float64)
    d = np.abs(x[:, None, 10:13] - alb[None]).max(2).min(1)
    assert (d == 0).all()
    assert ((x[:, 13] + x[:, 14]) == 1).all() and (x[:, 14] == 1).all()  # stylization enabled
    assert (x[:, 15:19].sum(1) == 1).all() and (x[:, 15] == 1).all()  # style index 0
    oh = x[:, 19:]
    assert (oh.sum(1) == 1).all() and set(np.unique(oh)) <= {0.0, 1.0}


def test_query_rows_both_layouts(sty, cornell):
    """Query rows are deterministic per seed and sample-major; the spherical layout encodes the
    same first hits as the reference layout."""
    sc, mats = cornell
    spp = 2
    xr, lr = sc.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, spp, D, layout=sty.scene.NRC_ROWS_REF, seed=9)
    xs, ls = sc.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, spp, D, layout=sty.scene.NRC_ROWS_SPHERICAL, seed=9)
    xr2, _ = sc.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, spp, D, layout=sty.scene.NRC_ROWS_REF, seed=9)
    assert xr.shape == (W * H * spp, 20 + D) and xs.shape == (W * H * spp, 11)
    assert bool((xr == xr2).all())
    xr, xs = xr.cpu().numpy().astype(np.float64), xs.cpu().numpy().astype(np.float64)
    assert (lr.cpu().numpy() == ls.cpu().numpy()).all()
    hit = xr[:, 9] > 0
    assert hit.mean() > 0.5
    assert (xr[~hit] == 0).all() and (xs[~hit] == 0).all()
    np.testing.assert_array_equal(xr[hit, :3], xs[hit, :3])

    def unsph(t, p):
        th, ph = t * np.pi, p * 2 * np.pi - np.pi
        return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)

    # theta = acos(z) loses digits near the poles (d theta = dz / sin theta): the allowance grows there
    for a, b in ((3, 3), (5, 6)):
        ref = xr[hit, b:b + 3] * 2 - 1
        sin_t = np.sqrt(np.maximum(1.0 - ref[:, 2] ** 2, 1e-12))
        err = np.abs(unsph(xs[hit, a], xs[hit, a + 1]) - ref).max(1)
        assert (err <= 2e-5 + 2e-7 / sin_t).all(), err.max()
    np.testing.assert_array_equal(xs[hit, 7:11], xr[hit, 9:13])
    assert (xr[hit, 19] == 1).all() and (xr[hit, 20:] == 0).all()  # depth one-hot 0


def test_bad_arguments_rejected(sty, cornell):
    import ctypes as C
    import torch
    sc, _ = cornell
    lib = sty.abi.lib()
    x = torch.empty((16, 11), device="cuda")
    y = torch.empty((16, 3), device="cuda")
    cnt = C.c_uint64()
    # query mode with too small a capacity, unknown layout, unknown mode
    assert lib.sty_nrc_samples(sc.h, 1, 1, 1, D, 0, x.data_ptr(), y.data_ptr(), 16, C.byref(cnt), None) != 0
    assert lib.sty_nrc_samples(sc.h, 0, 7, 1, D, 0, x.data_ptr(), y.data_ptr(), 16, C.byref(cnt), None) != 0
    assert lib.sty_nrc_samples(sc.h, 5, 1, 1, D, 0, x.data_ptr(), y.data_ptr(), 16, C.byref(cnt), None) != 0
    # training rows beyond the capacity are dropped, not written
    assert lib.sty_nrc_samples(sc.h, 0, 1, 1, D, 0, x.data_ptr(), y.data_ptr(), 16, C.byref(cnt), None) == 0
    assert cnt.value == 16


def _sees_light(sty, sc, spp=64):
    """Pixels whose footprint covers some of the emitter: any of `spp` first hits is on the light.
    Their radiance (17 where covered) dwarfs the rest of the image, so an edge pixel a few samples
    miss would otherwise dominate an MSE meant for the indirectly lit pixels."""
    _, le = sc.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, spp, D, seed=99)
    return (le.reshape(spp, H, W, 3).amax((0, 3)) > 0).cpu().numpy()


def _train_cache(sty, sc, precision, frames, iters, spp=4, lr=1e-2, seed=0):
    net = sty.nrc.NRC(sty.nrc.config(precision=precision, batch_size=1 << 14, learning_rate=lr, seed=77 + seed))
    for f in range(frames):
        x, y = sc.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, spp, D, seed=1000 + f + 10000 * seed)
        net.train(x, y, n_iters=iters, want_loss=False)
    return net


def _cache_image(sty, sc, net, xq):
    import torch
    spp = xq.shape[0] // (W * H)
    pred = net.inference(xq)
    pred = torch.where((xq[:, 7] > 0)[:, None], pred, torch.zeros_like(pred))
    return pred.reshape(spp, H, W, 3).mean(0).double().cpu().numpy()


def test_trained_cache_beats_cache_free_render(sty, cornell):
    """The learned part against the method without it: a cache trained online on tracer samples
    and read at the first hit (the depth-0 case of the reference's inference stage,
    nrc_pt.rs:877-965) has a lower image MSE against a 2048-spp render than the 1-spp cache-free
    render. BF16 (tensor-core training and inference) and FP32 caches reach the same MSE on the
    pixels off the emitter within 10 % (mean of two trainings each on this 32 x 32 image; the
    neural-cache benchmark holds the 5 % target on its workload). The pixels that see the light are
    left out of that comparison: a cache's error there is a few per cent of the light's radiance 17
    and varies from one training to the next, for either precision, by more than the precisions
    differ."""
    sc, _ = cornell
    gt, _ = sc.render(_self_only(sty, 4242, 256, repeats=8))
    gt = gt.cpu().numpy()
    xq, _ = sc.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, 4, D, seed=5)
    lit = _sees_light(sty, sc)

    def mse(im, mask=None):
        e = ((im - gt) ** 2).mean(2)
        return float(e.mean() if mask is None else e[mask].mean())

    pts = [sc.render(_self_only(sty, 10 + s, 1))[0].cpu().numpy() for s in range(8)]
    mse_pt = np.mean([mse(p) for p in pts])
    mse_pt_dark = np.mean([mse(p, ~lit) for p in pts])
    full, dark = {}, {}
    for prec in (sty.nrc.STY_NRC_FP32, sty.nrc.STY_NRC_BF16):
        f, d = [], []
        for seed in range(2):
            net = _train_cache(sty, sc, prec, frames=64, iters=8, seed=seed)
            im = _cache_image(sty, sc, net, xq)
            f.append(mse(im))
            d.append(mse(im, ~lit))
            net.close()
        full[prec], dark[prec] = float(np.mean(f)), float(np.mean(d))
    print(f"image mse: 1spp {mse_pt:.5f} (unlit {mse_pt_dark:.5f}); cache fp32 {full[0]:.5f} ({dark[0]:.5f}), "
          f"bf16 {full[1]:.5f} ({dark[1]:.5f})")
    for prec in (0, 1):
        assert full[prec] < 0.5 * mse_pt
        assert dark[prec] < 0.5 * mse_pt_dark
    assert abs(dark[1] - dark[0]) <= 0.10 * dark[0]
    assert abs(full[1] - full[0]) <= 0.15 * full[0]


def test_nrc_render_loop(sty, cornell):
    """The reference's NL-NRC loop (sty_nrc_render): training paths from random pixels, targets
    bootstrapped from the cache's own prediction at the next vertex, then the cache read at the
    first hit of every pixel. Against a 2048-spp render its image MSE is below the 1-spp cache-free
    render's; the whole loop is deterministic for a seed."""
    sc, _ = cornell
    gt, _ = sc.render(_self_only(sty, 4242, 256, repeats=8))
    gt = gt.cpu().numpy()
    mse_pt = np.mean([np.mean((sc.render(_self_only(sty, 10 + s, 1))[0].cpu().numpy() - gt) ** 2) for s in range(8)])
    imgs = []
    for _ in range(2):
        net = sty.nrc.NRC(sty.nrc.config(precision=sty.nrc.STY_NRC_BF16, batch_size=1 << 12, learning_rate=1e-2,
                                         seed=3))
        cfg = sty.scene.nrc_render_config(max_depth=D, training_iters=200, batches_per_iter=4, repeats=4, seed=7)
        film, st = sc.nrc_render(net, cfg)
        imgs.append(film.cpu().numpy())
        net.close()
    assert st.training_rows > 0 and st.inference_queries == 200 * D * W * H + 4 * W * H
    assert np.isfinite(st.last_loss)
    assert (imgs[0] == imgs[1]).all()
    mse = float(np.mean((imgs[0] - gt) ** 2))
    print(f"nrc render mse {mse:.5f} vs 1spp {mse_pt:.5f}")
    assert mse < 0.5 * mse_pt
    assert sty.abi.device_status() == 0


def test_nrc_render_rejects_wrong_cache(sty, cornell):
    sc, _ = cornell
    net = sty.nrc.NRC(sty.nrc.config(freqs=(4, 4, 4), batch_size=1 << 12, seed=1))  # 3 inputs, not 11
    with pytest.raises(sty.StyError):
        sc.nrc_render(net, sty.scene.nrc_render_config(max_depth=D, training_iters=1))
    net.close()


def test_nrc_render_final_gather(sty, cornell):
    """Final gathering (nrc_pt.rs:436-582, 969-1047): every Cornell-box first hit is rough, so each
    pixel splits at depth 0, gathers 16 rays whose hits the cache predicts, and keeps its own Le and
    direct light; against the 2048-spp render this beats both the 1-spp cache-free render and the
    cache read at the first hit, and it is deterministic."""
    sc, _ = cornell
    gt, _ = sc.render(_self_only(sty, 4242, 256, repeats=8))
    gt = gt.cpu().numpy()
    dk = ~_sees_light(sty, sc)
    mse_pt = np.mean([np.mean(((sc.render(_self_only(sty, 10 + s, 1))[0].cpu().numpy() - gt) ** 2)[dk])
                      for s in range(8)])
    out = {}
    for fg in (0, 16, 16):
        net = sty.nrc.NRC(sty.nrc.config(precision=sty.nrc.STY_NRC_BF16, batch_size=1 << 12, learning_rate=1e-2,
                                         seed=3))
        cfg = sty.scene.nrc_render_config(max_depth=D, training_iters=200, batches_per_iter=4, repeats=4, seed=7,
                                          final_gather=fg)
        film, st = sc.nrc_render(net, cfg)
        img = film.cpu().numpy()
        assert np.isfinite(img).all()
        out.setdefault(fg, []).append(img)
        net.close()
    assert (out[16][0] == out[16][1]).all()
    # on the pixels that do not see the emitter (final gathering improves the indirect light; at the
    # emitter's edge both renders carry the same coverage noise of the 4 camera samples)
    dark = ~_sees_light(sty, sc)
    m0 = float(np.mean(((out[0][0] - gt) ** 2)[dark]))
    m16 = float(np.mean(((out[16][0] - gt) ** 2)[dark]))
    print(f"final gather mse {m16:.5f}, first-hit cache {m0:.5f}, 1spp {mse_pt:.5f} (pixels off the emitter)")
    assert m16 < m0 and m16 < 0.5 * mse_pt
    assert sty.abi.device_status() == 0
