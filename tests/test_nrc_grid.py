"""The reference's NL-NRC network (sty_nrc_create_grid): composite encoding (hash grid + one-blob +
identity) and a ReLU MLP, against the FP64 oracle (oracle/nrc_grid.py + an emulation of the 16-bit
GEMM operands: BF16, or FP16 with tiny-cuda-nn's loss scale of 128 on the backward).

The forward reads FP16 copies of the tables (the emulation rounds them the same way); grid features
accumulate in FP32 and are rounded to BF16 like every GEMM operand, so outputs are compared to the
emulation statistically (98 % within 2e-3 of the output scale, all within 3e-2); gradients in norm
(MLP 1e-2, tables 2e-2 relative). Networks with 32, 64 or 128 hidden units run tensor-core
inference (tile encoder + on-chip MLP kernel); `layered=True` forces the layer-by-layer GEMM path."""
import numpy as np
import pytest

import oracle.nrc as onrc
import oracle.nrc_grid as og

# a small network with dense and hashed levels
SMALL = dict(max_depth=5, hidden_layers=2, hidden_units=32, grid_levels=6, grid_features=2, log2_table=12,
             base_resolution=4, per_level_scale=2.0, blob_dims=7, blob_bins=4)


def _geo(c):
    return og.level_geometry(c["grid_levels"], c["log2_table"], c["base_resolution"], c["per_level_scale"])


def test_oracle_geometry_teaser():
    geo, offs, total = og.level_geometry(22, 19, 16, 2.0)
    assert [g[3] for g in geo[:4]] == [True, True, True, False]
    assert [g[2] for g in geo[:4]] == [16 ** 3, 32 ** 3, 64 ** 3, 1 << 19]
    assert total == 16 ** 3 + 32 ** 3 + 64 ** 3 + 19 * (1 << 19)


def test_oracle_grid_backward_is_the_gradient():
    c = SMALL
    _, _, total = _geo(c)
    rng = np.random.default_rng(0)
    x = rng.random((40, 3))
    t = rng.uniform(-1, 1, (total, c["grid_features"]))
    d = rng.normal(size=(40, c["grid_levels"] * c["grid_features"]))
    args = (c["grid_levels"], c["grid_features"], c["log2_table"], c["base_resolution"], c["per_level_scale"])
    g = og.grid_backward(x, d, *args, total)
    f0 = float((og.grid_forward(x, t, *args) * d).sum())
    for idx in rng.choice(np.flatnonzero(np.abs(g).sum(1)), 10, replace=False):
        e = np.zeros_like(t)
        e[idx, 1] = 1.0
        f1 = float((og.grid_forward(x, t + e, *args) * d).sum())  # the features are linear in the tables
        assert f1 - f0 == pytest.approx(g[idx, 1], rel=1e-9, abs=1e-12)


def test_oracle_oneblob():
    b = og.oneblob(np.array([[0.5, 0.3, 0.0]]), 4).reshape(3, 4)
    assert b[0].sum() == pytest.approx(0.9545, abs=1e-3)  # +-2 sigma inside [0, 1]
    assert b[0][1] == pytest.approx(b[0][2]) and b[0][0] == pytest.approx(b[0][3])
    assert b[2][0] > b[2][1] > b[2][2]


def _net(sty, seed=3, batch=1024, **kw):
    c = dict(SMALL)
    c.update(kw)
    return sty.nrc.NRC(sty.nrc.grid_config(batch_size=batch, seed=seed, **c)), c


def _split(p, c):
    """MLP weights (list of [out, in] matrices) and tables from the flat parameters."""
    E = c["grid_levels"] * c["grid_features"] + c["blob_dims"] * c["blob_bins"] + (20 + c["max_depth"] - 3 - c["blob_dims"])
    Ep = (E + 15) // 16 * 16
    H, L = c["hidden_units"], c["hidden_layers"]
    mats, o = [], 0
    for l in range(L):
        k = Ep if l == 0 else H
        mats.append(p[o:o + H * k].reshape(H, k))
        o += H * k
    mats.append(p[o:o + 3 * H].reshape(3, H))
    o += 3 * H
    return mats, p[o:].reshape(-1, c["grid_features"]), Ep


def _emulate(p, c, x):
    r16 = onrc.fp16_round if c.get("fp16") else onrc.bf16_round
    mats, tables, Ep = _split(p.astype(np.float64), c)
    tables = tables.astype(np.float16).astype(np.float64)
    enc = og.encode(x, tables, c["grid_levels"], c["grid_features"], c["log2_table"], c["base_resolution"],
                    c["per_level_scale"], c["blob_dims"], c["blob_bins"], Ep)
    mb = [r16(m) for m in mats]
    acts = [r16(enc)]
    h = acts[0]
    for l in range(c["hidden_layers"]):
        h = r16(np.maximum(h @ mb[l].T, 0.0))
        acts.append(h)
    return h @ mb[-1].T, acts, mb, enc


def _rows(rng, n, c):
    x = rng.random((n, 20 + c["max_depth"]))
    x[:, 10:] = (x[:, 10:] > 0.5)  # one-hot-like flag / depth columns
    return x


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("fp16", [False, True], ids=["bf16", "fp16"])
def test_grid_inference_matches_emulation(sty, cuda, fp16):
    net, c = _net(sty, fp16=fp16)
    p = net.save_params().astype(np.float64)
    # spread the tables so the encoding matters
    mats, tables, _ = _split(p, c)
    rng = np.random.default_rng(1)
    p[len(p) - tables.size:] = rng.uniform(-0.5, 0.5, tables.size)
    net.load_params(p.astype(np.float32))
    p = p.astype(np.float32).astype(np.float64)
    x = _rows(rng, 3000, c)
    out = net.inference(_dev(x)).cpu().numpy()
    ref, _, _, _ = _emulate(p, c, x)
    scale = np.abs(ref).max()
    err = np.abs(out - ref)
    assert np.isfinite(out).all()
    assert np.mean(err <= 2e-3 * scale) >= 0.98, np.mean(err > 2e-3 * scale)
    assert err.max() <= 3e-2 * scale
    assert sty.abi.device_status() == 0


TEASER_SHAPE = dict(max_depth=12, hidden_units=128, hidden_layers=5, grid_levels=22, grid_features=4,
                    log2_table=14, base_resolution=16)


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(), dict(hidden_units=64, hidden_layers=3, grid_levels=8, grid_features=4),
                                dict(hidden_units=128, hidden_layers=2, grid_levels=5, grid_features=8),
                                TEASER_SHAPE], ids=["h32f2", "h64f4", "h128f8", "teaser-shape"])
def test_grid_tc_matches_layered(sty, cuda, kw):
    """Tensor-core inference (tile encoder + every layer on chip) against the layer-by-layer GEMM
    path and the emulation, on ragged row counts (partial tiles, fewer rows than one tile)."""
    fused, c = _net(sty, seed=9, **kw)
    layered, _ = _net(sty, seed=9, layered=True, **kw)
    p = fused.save_params().astype(np.float64)
    rng = np.random.default_rng(3)
    _, tables, _ = _split(p, c)
    p[len(p) - tables.size:] = rng.uniform(-0.5, 0.5, tables.size)
    p32 = p.astype(np.float32)
    fused.load_params(p32)
    layered.load_params(p32)
    for n in (1, 127, 128, 1000, 5000):
        x = _rows(rng, n, c)
        a = fused.inference(_dev(x)).cpu().numpy()
        b = layered.inference(_dev(x)).cpu().numpy()
        ref, _, _, _ = _emulate(p32.astype(np.float64), c, x)
        scale = np.abs(ref).max()
        assert a.shape == (n, 3) and np.isfinite(a).all()
        for out in (a, b):
            err = np.abs(out - ref)
            assert np.mean(err <= 2e-3 * scale) >= 0.98, (n, np.mean(err > 2e-3 * scale))
            assert err.max() <= 3e-2 * scale, (n, err.max() / scale)
        assert np.abs(a - b).max() <= 3e-2 * scale
    assert sty.abi.device_status() == 0
    fused.close()
    layered.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(), dict(fp16=True), dict(hidden_units=128, grid_levels=12, grid_features=4),
                                dict(hidden_units=128, grid_levels=12, grid_features=4, fp16=True)],
                         ids=["bf16", "fp16", "bf16-h128", "fp16-h128"])
def test_grid_gradient_matches_emulation(sty, cuda, kw):
    """The full parameter gradient (tensor-core GEMMs forward, input and weight gradients reduced over
    the batch in a fixed order; table gradient by atomics) against the emulation of the same 16-bit
    operands; deterministic for the MLP part."""
    net, c = _net(sty, seed=5, **kw)
    p = net.save_params().astype(np.float64)
    rng = np.random.default_rng(2)
    mats, tables, Ep = _split(p, c)
    p[len(p) - tables.size:] = rng.uniform(-0.5, 0.5, tables.size)
    net.load_params(p.astype(np.float32))
    p = p.astype(np.float32).astype(np.float64)
    B = 512
    x = _rows(rng, B, c)
    t = rng.random((B, 3)) + 0.1
    g, loss = net.gradient(_dev(x), _dev(t))
    g = g.cpu().numpy().astype(np.float64)
    # emulated backward: 16-bit loss gradient (times the loss scale S) and layer gradients, sums in
    # FP64, the weight and encoding gradients divided by S
    r16 = onrc.fp16_round if c.get("fp16") else onrc.bf16_round
    S = 128.0 if c.get("fp16") else 1.0
    pred, acts, mb, enc = _emulate(p, c, x)
    den = pred * pred + 0.01
    gp = r16(S * 2.0 * (pred - t) / den / (B * 3))
    grads = [None] * (c["hidden_layers"] + 1)
    grads[-1] = gp.T @ acts[-1] / S
    dh = gp @ mb[-1]
    for l in range(c["hidden_layers"] - 1, -1, -1):
        dp = r16(dh * (acts[l + 1] > 0))
        grads[l] = dp.T @ acts[l] / S
        dh = dp @ mb[l]
    dh = dh / S
    ng = c["grid_levels"] * c["grid_features"]
    _, _, total = _geo(c)
    gt = og.grid_backward(x[:, :3], dh[:, :ng], c["grid_levels"], c["grid_features"], c["log2_table"],
                          c["base_resolution"], c["per_level_scale"], total)
    ref_mlp = np.concatenate([m.reshape(-1) for m in grads])
    n_mlp = ref_mlp.size
    assert np.linalg.norm(g[:n_mlp] - ref_mlp) <= 1e-2 * np.linalg.norm(ref_mlp)
    assert np.linalg.norm(g[n_mlp:] - gt.reshape(-1)) <= 2e-2 * np.linalg.norm(gt)
    assert loss == pytest.approx(float(((pred - t) ** 2 / den).mean()), rel=1e-2)
    g2, _ = net.gradient(_dev(x), _dev(t))
    assert np.array_equal(g2.cpu().numpy()[:n_mlp], g[:n_mlp].astype(np.float32))  # fixed-order reductions
    net.close()


def test_oracle_adam_sparse_rule():
    """Table entries with a zero gradient keep weight, moments and step count; the others use their
    own step count in the bias correction."""
    n_mlp = 2
    w = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    z = np.zeros(5)
    g = np.array([0.5, 0.0, 0.25, 0.0, -1.0])
    w1, m1, v1, ts = og.adam_step(w, z, z, g, np.zeros(3), n_mlp, t=1, lr=0.1)
    assert w1[1] == 2.0 - 0.0 and m1[1] == 0.0  # MLP weight with a zero gradient still steps (by 0)
    assert w1[3] == 4.0 and m1[3] == 0.0 and list(ts) == [1, 0, 1]
    assert w1[0] == pytest.approx(1.0 - 0.1) and w1[4] == pytest.approx(5.0 + 0.1)  # |step| = lr at t = 1
    # second step: entry 3 gets its first update (t_p = 1) while the MLP is at t = 2
    g2 = np.array([0.5, 0.0, 0.0, 2.0, 0.0])
    w2, m2, v2, ts2 = og.adam_step(w1, m1, v1, g2, ts, n_mlp, t=2, lr=0.1)
    assert w2[3] == pytest.approx(4.0 - 0.1) and w2[2] == w1[2] and w2[4] == w1[4] and list(ts2) == [1, 1, 1]


@pytest.mark.gpu
def test_grid_optimiser_matches_oracle(sty, cuda):
    """One training step on a batch of identical rows (so batch sampling cannot matter) against the
    oracle's Adam on the same gradient; then a step on another row, after which the table entries
    only the first row touched are bit-identical (a dense Adam would move them by momentum)."""
    c = dict(SMALL)
    lr = 1e-2
    net = sty.nrc.NRC(sty.nrc.grid_config(batch_size=128, seed=4, learning_rate=lr, **c))
    rng = np.random.default_rng(8)
    xa, xb = _rows(rng, 1, c), _rows(rng, 1, c)
    ta, tb = rng.random((1, 3)) + 0.2, rng.random((1, 3)) + 0.2
    XA, TA = _dev(np.repeat(xa, 128, 0)), _dev(np.repeat(ta, 128, 0))
    XB, TB = _dev(np.repeat(xb, 128, 0)), _dev(np.repeat(tb, 128, 0))
    p0 = net.save_params().astype(np.float64)
    n_tab = _split(p0, c)[1].size
    n_mlp = p0.size - n_tab
    ga = net.gradient(XA, TA)[0].cpu().numpy().astype(np.float64)
    net.train(XA, TA, 1)
    p1 = net.save_params().astype(np.float64)
    z = np.zeros_like(p0)
    w1, m1, v1, ts1 = og.adam_step(p0, z, z, ga, np.zeros(n_tab), n_mlp, t=1, lr=lr)
    touched_a = ga[n_mlp:] != 0
    assert touched_a.sum() > 0 and (~touched_a).sum() > 0
    np.testing.assert_allclose(p1, w1, rtol=2e-5, atol=1e-7)
    gb = net.gradient(XB, TB)[0].cpu().numpy().astype(np.float64)
    net.train(XB, TB, 1)
    p2 = net.save_params().astype(np.float64)
    w2, _, _, _ = og.adam_step(w1, m1, v1, gb, ts1, n_mlp, t=2, lr=lr)
    only_a = touched_a & (gb[n_mlp:] == 0)
    assert only_a.sum() > 0
    assert np.array_equal(p2[n_mlp:][only_a], p1[n_mlp:][only_a])
    np.testing.assert_allclose(p2, w2, rtol=5e-5, atol=1e-7)
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("fp16", [False, True], ids=["bf16", "fp16"])
def test_grid_training_reduces_loss(sty, cuda, fp16):
    net, c = _net(sty, seed=7, batch=4096, learning_rate=1e-2, fp16=fp16)
    rng = np.random.default_rng(4)
    x = _rows(rng, 1 << 15, c)
    tgt = np.stack([0.5 + 0.4 * np.sin(4 * x[:, 0] + 3 * x[:, 1]), 0.3 + 0.3 * x[:, 2] * x[:, 4],
                    0.2 + 0.2 * np.cos(5 * x[:, 1]) + 0.1 * x[:, 12]], 1)
    xd, td = _dev(x), _dev(tgt)
    first = net.train(xd, td, 1)
    for _ in range(6):
        last = net.train(xd, td, 50)
    assert last < 0.1 * first, (first, last)


@pytest.mark.gpu
def test_grid_teaser_network(sty, cuda):
    """The teaser's configuration (configs/teaser/nl-nrc.json): 22 x 4 hash grid on 2^19-entry
    tables, 5 x 128 MLP, max depth 12 (32 inputs), batch 2^16."""
    net = sty.nrc.NRC(sty.nrc.grid_config(max_depth=12, seed=11))
    assert net.param_count() == 144 * 128 + 4 * 128 * 128 + 3 * 128 + 4 * (16 ** 3 + 32 ** 3 + 64 ** 3 + 19 * (1 << 19))
    rng = np.random.default_rng(6)
    x = _dev(_rows(rng, 1 << 17, dict(max_depth=12)))
    t = _dev(rng.random((1 << 17, 3)))
    l0 = net.train(x, t, 2)
    y = net.inference(x).cpu().numpy()
    assert np.isfinite(l0) and np.isfinite(y).all()
    assert sty.abi.device_status() == 0
    net.close()


@pytest.mark.gpu
def test_grid_network_in_the_nrc_render(sty, cuda):
    """The reference's network inside the NL-NRC loop (rows in the reference layout): the cache
    render of the Cornell box beats the 1-spp cache-free render against a 2048-spp render."""
    W = H = 32
    D = 4
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    so = lambda seed, b, r=1: sty.scene.render_config(max_depth=D, branch=b, repeats=r, radius_scale=(1e-4,),  # noqa: E731
                                                       reuse=(8,), smis=False, seed=seed)
    gt = sc.render(so(4242, 256, 8))[0].cpu().numpy()
    mse_pt = np.mean([np.mean((sc.render(so(10 + s, 1))[0].cpu().numpy() - gt) ** 2) for s in range(4)])
    net = sty.nrc.NRC(sty.nrc.grid_config(max_depth=D, batch_size=1 << 12, hidden_units=64, grid_levels=8,
                                          grid_features=2, log2_table=16, learning_rate=1e-2, seed=2))
    film, st = sc.nrc_render(net, sty.scene.nrc_render_config(max_depth=D, training_iters=200, batches_per_iter=4,
                                                               repeats=4, seed=7))
    img = film.cpu().numpy()
    mse = float(np.mean((img - gt) ** 2))
    print(f"grid-network nrc render mse {mse:.5f} vs 1spp {mse_pt:.5f}")
    assert np.isfinite(img).all() and st.training_rows > 0
    # the table gradient is summed with float atomics, so training is not bit-reproducible; over 14
    # runs the ratio to the 1-spp error spread from 0.31 to 0.59
    assert mse < 0.75 * mse_pt
    net.close()
