"""Reference-mode NL-PF (world-space grid, clustering, SMIS).

CPU part: the oracle is pinned by analytic single-neighbour cases, a brute-force neighbour count
and clustering invariants. GPU part: the CUDA path against the oracle on the same buffers --
neighbour counts, cluster ids and reservoir RNG states bit-exact, radiance within 1e-5 relative
(FP32 kernel vs FP64 oracle)."""
import math

import numpy as np
import pytest

from conftest import rel_err

TOL = 1e-5


def _setup(sty, n=3000, seed=0, **kw):
    arr = sty.synth.ref_vertices(n, seed, **kw)
    pfr = sty.pf_ref
    mats = pfr.materials([
        (pfr.STY_MAT_DIFFUSE, (0.75, 0.75, 0.75), 0.0, (0, -1, 1, -1)),
        (pfr.STY_MAT_DIFFUSE, (0.63, 0.065, 0.05), 0.0, (1, 1, -1, -1)),
        (pfr.STY_MAT_GGX, (0.9, 0.8, 0.6), 0.3, (-1, 0, -1, 1)),
    ])
    a = sty.abi
    progs = pfr.programs([
        a.style_program([a.ramp_smooth(20.0, [0.05, 0.3, 0.9], [(0.1, 0.1, 0.2), (0.5, 0.4, 0.3), (1.2, 1.1, 0.9)])]),
        a.style_program([a.sat_rex(0.4)]),
    ])
    rng = np.zeros((n, 2), dtype=np.uint64)
    rng[:, 0] = np.arange(n, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    rng[:, 1] = (np.arange(n, dtype=np.uint64) << np.uint64(1)) | np.uint64(1)
    return arr, mats, progs, rng


# ---------------------------------------------------------------- CPU: pinning the oracle
def test_single_vertex_analytic(orc, sty):
    """One active vertex: its only neighbour is itself. direct = f L w / pdf_light with the balance
    MIS weight; SMIS indirect = f L mis / pdf_self (lm_path_filtering.rs:839-944)."""
    arr, mats, progs, rng = _setup(sty, n=50, seed=3)
    arr["active"][:] = 0
    i = 7
    arr["active"][i] = 1
    arr["material"][i] = 0
    arr["flags"][i] = 1  # stylization disabled: raw radiance comes out
    arr["dir_pdf"][i] = 0.8
    prm = sty.pf_ref.RefParams(depth=1, radius=0.2, reuse=8)
    st, out, nb, _, _ = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    assert st == 0 and nb[i] == 1 and nb.sum() == 1
    ns, wo = arr["ns"][:, i].astype(float), arr["wo"][:, i].astype(float)
    alb = 0.75

    def lam(wi):
        ci = float(np.dot(wi, ns))
        return alb / math.pi * abs(ci), abs(ci) / math.pi

    f, pb = lam(arr["dir_wi"][:, i].astype(float))
    w = 0.8 / (0.8 + pb)
    direct = f * arr["dir_l"][:, i].astype(float) * w / 0.8
    f2, p2 = lam(arr["ind_wi"][:, i].astype(float))
    indirect = f2 * arr["in_next"][:, i].astype(float) * float(arr["ind_mis"][i]) / p2 \
        if np.any(arr["ind_wi"][:, i]) else 0.0
    ref = arr["le"][:, i].astype(float) + direct + indirect
    assert np.allclose(out[:, i], ref, rtol=1e-6)
    assert (out[:, np.arange(50) != i] == 0).all()


def test_neighbour_counts_brute_force(orc, sty):
    arr, mats, progs, rng = _setup(sty, n=800, seed=5)
    prm = sty.pf_ref.RefParams(depth=1, radius=0.15, reuse=4, disable_flag_check=True)
    st, out, nb, _, rng_after = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    assert st == 0
    p = arr["p"].T.astype(np.float32)
    act = arr["active"].astype(bool)
    for i in np.flatnonzero(act)[:200]:
        d = p[act] - p[i]
        dist = np.sqrt(((d[:, 0] * d[:, 0]) + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2], dtype=np.float32)
        assert nb[i] == int((dist <= np.float32(0.15)).sum())
    # reservoir draws happen exactly when the count exceeds the capacity
    moved = (rng_after[:, 0] != rng[:, 0])
    assert (moved == (nb > 4)).all()


def test_clustering_invariants(orc, sty):
    arr, mats, progs, rng = _setup(sty, n=2000, seed=9)
    prm = sty.pf_ref.RefParams(depth=2, radius=0.12, reuse=6, cluster=True)
    st, out, nb, cid, _ = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    assert st == 0
    act = arr["active"].astype(bool)
    assert (cid[~act] == 0xFFFFFFFF).all() and (cid[act] != 0xFFFFFFFF).all()
    centers = np.unique(cid[act])
    assert (cid[centers] == centers).all()
    p = arr["p"].T.astype(np.float32)
    for c in centers:
        members = np.flatnonzero(cid == c)
        assert len(members) <= prm.reuse + 1
        d = p[members] - p[c]
        assert (np.sqrt((d * d).sum(1)) <= 0.12 * (1 + 1e-6)).all()
    # deterministic
    st2, out2, nb2, cid2, _ = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    assert (cid2 == cid).all() and (nb2 == nb).all() and (out2 == out).all()


def test_iteration_cap_reports_error(orc, sty):
    arr, mats, progs, rng = _setup(sty, n=1500, seed=2)
    prm = sty.pf_ref.RefParams(depth=1, radius=0.3, reuse=2, cluster=True, max_cluster_rounds=1)
    st, *_ = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    assert st == sty.STY_ERR_ITER_LIMIT


# ---------------------------------------------------------------- GPU parity
def _gpu(sty, arr, mats, progs, rng, prm, n_progs=2):
    import torch
    dev = sty.pf_ref.to_device({k: v for k, v in arr.items() if k != "in_next"})
    in_next = torch.from_numpy(arr["in_next"]).cuda()
    n = arr["active"].shape[0]
    r = torch.from_numpy(rng.copy()).cuda()
    nb = torch.zeros(n, dtype=torch.int32, device="cuda")
    cid = torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx = sty.pf_ref.RefContext(n, prm.table_size)
    out = ctx.filter(dev, prm, mats, progs, n_progs, r, in_next=in_next, neighbours=nb, cluster_id=cid)
    torch.cuda.synchronize()
    ctx.close()
    return (out.cpu().numpy(), nb.cpu().numpy().view(np.uint32), cid.cpu().numpy().view(np.uint32),
            r.cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("cluster", [False, True])
@pytest.mark.parametrize("smis", [True, False])
@pytest.mark.parametrize("reuse", [1, 3, 4, 64])
def test_ref_filter_matches_oracle(sty, orc, cuda, cluster, smis, reuse):
    arr, mats, progs, rng = _setup(sty, n=6000, seed=11 + reuse)
    prm = sty.pf_ref.RefParams(depth=1, radius=0.08, reuse=reuse, smis=smis, cluster=cluster)
    st, ref_out, ref_nb, ref_cid, ref_rng = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng,
                                                              in_next=arr["in_next"])
    assert st == 0
    out, nb, cid, r = _gpu(sty, arr, mats, progs, rng, prm)
    assert (nb == ref_nb).all()
    if cluster:
        assert (cid == ref_cid).all()
    assert (r == ref_rng).all()
    act = arr["active"].astype(bool)
    assert (out[:, ~act] == 0).all()
    err = rel_err(out[:, act], ref_out[:, act], 1e-4)
    assert err.max() < TOL, f"max rel err {err.max():.3e}"


@pytest.mark.gpu
def test_ref_filter_flags_and_depth0(sty, orc, cuda):
    arr, mats, progs, rng = _setup(sty, n=4000, seed=21, p_flags=0.5)
    for prm in (sty.pf_ref.RefParams(depth=0, radius=0.1, reuse=32, no_first_hit_stylization=True),
                sty.pf_ref.RefParams(depth=0, radius=0.1, reuse=32, disable_flag_check=True),
                sty.pf_ref.RefParams(depth=3, radius=0.1, reuse=32, pmin=(-8, -8, -8), pmax=(8, 8, 8),
                                     table_size=(1 << 20) + 7)):
        st, ref_out, ref_nb, _, _ = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
        assert st == 0
        out, nb, _, _ = _gpu(sty, arr, mats, progs, rng, prm)
        assert (nb == ref_nb).all()
        act = arr["active"].astype(bool)
        assert rel_err(out[:, act], ref_out[:, act], 1e-4).max() < TOL


@pytest.mark.gpu
def test_ref_filter_iteration_cap(sty, cuda):
    arr, mats, progs, rng = _setup(sty, n=1500, seed=2)
    prm = sty.pf_ref.RefParams(depth=1, radius=0.3, reuse=2, cluster=True, max_cluster_rounds=1)
    with pytest.raises(sty.StyError) as ei:
        _gpu(sty, arr, mats, progs, rng, prm)
    assert ei.value.status == sty.STY_ERR_ITER_LIMIT


def test_oracle_select_matches_full(orc, sty):
    """Filtering a selection of vertices gives exactly the full run's values there (each vertex draws
    from its own PCG32 stream, the grid is built from every vertex)."""
    arr, mats, progs, rng = _setup(sty, n=2500, seed=31)
    prm = sty.pf_ref.RefParams(depth=1, radius=0.1, reuse=16, smis=True)
    st, out, nb, _, r = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"])
    sel = np.zeros(2500, bool)
    sel[np.random.default_rng(1).choice(2500, 300, replace=False)] = True
    st2, out2, nb2, _, r2 = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"], select=sel)
    assert st == st2 == 0
    np.testing.assert_array_equal(out2[:, sel], out[:, sel])
    np.testing.assert_array_equal(nb2[sel], nb[sel])
    np.testing.assert_array_equal(r2[sel], r[sel])
    assert (out2[:, ~sel] == 0).all() and (r2[~sel] == rng[~sel]).all()


@pytest.mark.gpu
def test_ref_filter_full_vertex_count(sty, orc, cuda):
    """A depth of the end-to-end render's size (256x256 pixels x 16 paths = 1 048 576 vertex slots,
    radius 0.05, reuse 64, SMIS): 2000 sampled vertices against the oracle -- neighbour counts and
    reservoir RNG states bit-exact, radiance within 1e-5."""
    n = 1 << 20
    arr, mats, progs, rng = _setup(sty, n=n, seed=41)
    prm = sty.pf_ref.RefParams(depth=1, radius=0.05, reuse=64, smis=True, table_size=(1 << 22) + 15)
    out, nb, _, r = _gpu(sty, arr, mats, progs, rng, prm)
    sel = np.zeros(n, bool)
    sel[np.random.default_rng(2).choice(n, 2000, replace=False)] = True
    sel &= arr["active"].astype(bool)
    st, ref_out, ref_nb, _, ref_rng = orc.pf_ref_filter(arr, prm.c(), mats, progs, 2, rng, in_next=arr["in_next"],
                                                        select=sel)
    assert st == 0 and sel.sum() > 1500
    assert (nb[sel] == ref_nb[sel]).all()
    assert np.median(nb[sel]) > 100  # a dense neighbourhood, as in the render
    assert (r[sel] == ref_rng[sel]).all()
    err = rel_err(out[:, sel], ref_out[:, sel], 1e-4)
    assert err.max() < TOL, f"max rel err {err.max():.3e}"
