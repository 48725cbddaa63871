"""Wavefront tracer and the end-to-end NL-PF render.

- first hits: GPU BVH traversal vs a brute-force oracle over every triangle, same watertight test:
  triangle ids and distances bit-exact on identical rays (camera rays and random interior rays);
- self-only filtering: the full pipeline (trace, emitter MIS, NEE, reference-mode filter with and
  without SMIS, splat) converges to an independent FP64 CPU path tracer on the Cornell box;
- the Cornell box renders deterministically and finitely with and without style nodes."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _camera_rays(cam, n_per_pixel=2, seed=0):
    """Pinhole rays through jittered pixel positions (float32), as 8-float records."""
    rng = np.random.default_rng(seed)
    W, H = cam.width, cam.height
    eye = np.array(cam.eye[:], np.float32)
    f = np.array(cam.target[:], np.float32) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, np.array(cam.up[:], np.float32))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    th = np.float32(np.tan(np.radians(cam.fov_y) / 2))
    ys, xs = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    xs = np.repeat(xs.reshape(-1), n_per_pixel).astype(np.float32) + rng.random(W * H * n_per_pixel, np.float32)
    ys = np.repeat(ys.reshape(-1), n_per_pixel).astype(np.float32) + rng.random(W * H * n_per_pixel, np.float32)
    sx = (2 * xs / W - 1) * th * (W / H)
    sy = (1 - 2 * ys / H) * th
    d = f[None] + sx[:, None] * r[None] + sy[:, None] * u[None]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((d.shape[0], 8), np.float32)
    rays[:, 0:3] = eye
    rays[:, 3:6] = d
    rays[:, 7] = 1e20
    return rays


def test_first_hits_bit_exact(sty, cuda):
    import torch
    pos, mids, mats, cam = sty.scene.cornell_box(48, 40)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    rays = _camera_rays(cam)
    rng = np.random.default_rng(1)
    m = 20000
    inner = np.zeros((m, 8), np.float32)
    inner[:, 0:3] = rng.uniform(0.02, 0.98, (m, 3))
    dd = rng.normal(size=(m, 3))
    inner[:, 3:6] = dd / np.linalg.norm(dd, axis=1, keepdims=True)
    inner[:, 7] = 1e20
    allr = np.concatenate([rays, inner])
    prim, t, b = sc.closest_hit(torch.from_numpy(allr).cuda())
    torch.cuda.synchronize()
    rp, rt, rb = oracle.closest_hit(pos, allr)
    gp = prim.cpu().numpy().view(np.uint32)
    assert (gp == rp).all(), f"{(gp != rp).sum()} first-hit ids differ"
    assert (t.cpu().numpy() == rt).all()
    assert (b.cpu().numpy() == rb).all()
    assert (rp[: len(rays)] != 0xFFFFFFFF).mean() > 0.99  # the box is closed except behind the camera


@pytest.mark.parametrize("smis", [True, False])
def test_self_only_render_matches_cpu_path_tracer(sty, cuda, smis):
    """With a filter radius so small that every vertex only reuses itself and no style nodes, the
    NL-PF estimator of the reference is the textbook NEE + MIS path tracer (emitters are black), so
    the full GPU pipeline must converge to the independent FP64 CPU path tracer."""
    W = H = 32
    D = 4
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    cfg = sty.scene.render_config(max_depth=D, branch=64, repeats=4, radius_scale=(1e-4,), reuse=(8,), smis=smis,
                                  seed=5)
    film, nv = sc.render(cfg)
    img = film.cpu().numpy()
    alb = np.array([m.albedo[:] for m in mats], np.float32)
    em = np.array([m.emission[:] for m in mats], np.float32)
    camv = list(cam.eye) + list(cam.target) + list(cam.up) + [cam.fov_y, W, H, cam.filter_radius]
    ref = oracle.path_trace(pos, mids, alb, em, camv, 256, D, seed=11)
    assert np.isfinite(img).all()
    m_img, m_ref = img.mean(), ref.mean()
    assert abs(m_img - m_ref) < 0.02 * m_ref, (m_img, m_ref)
    bi = img.reshape(4, 8, 4, 8, 3).mean((1, 3))
    br = ref.reshape(4, 8, 4, 8, 3).mean((1, 3))
    rel = np.abs(bi - br) / np.maximum(br, 0.05 * m_ref)
    assert rel.max() < 0.15, rel.max()


def test_cornell_render_deterministic(sty, cuda):
    a = sty.abi
    pos, mids, mats, cam = sty.scene.cornell_box(64, 48, style=(0, -1, -1, -1))
    sc = sty.scene.Scene(pos, mids, mats, cam)
    progs = [a.style_program([a.toon(0.2)])]
    for cluster in (False, True):
        cfg = sty.scene.render_config(max_depth=4, branch=4, radius_scale=(5.0,), reuse=(32,), cluster=cluster, seed=7)
        f1, n1 = sc.render(cfg, progs)
        f2, n2 = sc.render(cfg, progs)
        i1, i2 = f1.cpu().numpy(), f2.cpu().numpy()
        assert n1 == n2 and n1 > 64 * 48 * 4
        assert np.isfinite(i1).all() and (i1 == i2).all()
        assert 0.05 < i1.mean() < 5.0
    assert sty.abi.device_status() == 0


def test_room_scene_renders(sty, cuda):
    """The interior workload scene: light from the corridor emitter reaches the room only through
    the door gap; the NL-PF and NL-NRC renders of it are finite, lit, and deterministic."""
    pos, mids, mats, cam = sty.scene.room_with_door(48, 27, cell=0.2)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    a = sty.abi
    progs = [a.style_program([a.toon(0.2, depth_mask=0b11)])]
    cfg = sty.scene.render_config(max_depth=6, branch=8, radius_scale=(1.0,), reuse=(16,), seed=2)
    f1, nv = sc.render(cfg, progs)
    f2, _ = sc.render(cfg, progs)
    img = f1.cpu().numpy()
    assert nv > 0 and np.isfinite(img).all() and img.mean() > 1e-3
    assert (f1 == f2).all()
    net = sty.nrc.NRC(sty.nrc.config(batch_size=1 << 12, seed=2))
    film, st = sc.nrc_render(net, sty.scene.nrc_render_config(max_depth=6, training_iters=8, batches_per_iter=2),
                             progs)
    im = film.cpu().numpy()
    assert np.isfinite(im).all() and st.training_rows > 0
    net.close()
    assert sty.abi.device_status() == 0
