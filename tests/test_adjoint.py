"""Adjoint of the screen-space NL-PF filter + smoothed ramp style node (36 parameters).

CPU: the oracle's analytic FP64 adjoint against FP64 central finite differences (h = 1e-4).
GPU: the CUDA adjoint (FP32, weights recomputed in the backward) against the FP64 finite
differences and the FP64 analytic adjoint, within 1e-4 relative (per parameter, relative to the
gradient's largest entry of the same group for entries near zero)."""
import numpy as np
import pytest

import oracle

H_FD = 1e-4


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(36)
    p[0] = 50.0 / 10.0  # sharpness (scaled down so the small test image has non-saturated sigmoids)
    p[1:9] = np.sort(rng.uniform(0.05, 1.2, 8))
    p[9:33] = np.sort(rng.uniform(0.0, 1.0, 24))
    p[33:36] = [3.0, 0.6, 0.3]
    return p


def _case(sty, W=24, H=16, S=4, seed=5):
    planes, valid = sty.synth.records(W, H, S, 1, seed=seed)
    rec = sty.pf.host_records(planes, valid, W, H, S, 1)
    p = _params(seed)
    rng = np.random.default_rng(seed + 1)
    # target = image rendered with a perturbed parameter vector (Gaussian sigma 0.05)
    pt = p + rng.normal(0.0, 0.05, 36) * np.abs(p)
    pt[33:36] = np.abs(pt[33:36])
    return planes, valid, rec, p, pt


def _target(orc, rec, pt, R, W, H):
    """Target image: the FP64 render with the perturbed parameter vector."""
    return orc.pf_adjoint_image(rec, 0, R, pt, 8)


def _fd(orc, rec, p, R, target):
    g = np.zeros(36)
    for k in range(36):
        e = np.zeros(36)
        e[k] = H_FD
        g[k] = (orc.pf_adjoint_loss(rec, 0, R, p + e, 8, target) -
                orc.pf_adjoint_loss(rec, 0, R, p - e, 8, target)) / (2 * H_FD)
    return g


def _close(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.maximum(np.abs(b), 1e-3 * np.abs(b).max())
    return (np.abs(a - b) / scale).max()


def test_oracle_adjoint_matches_fd(sty):
    W, H, R = 12, 8, 3
    planes, valid, rec, p, pt = _case(sty, W, H, 4, seed=5)
    target = _target(oracle, rec, pt, R, W, H)
    loss, g = oracle.pf_adjoint(rec, 0, R, p, 8, target)
    assert loss > 0
    fd = _fd(oracle, rec, p, R, target)
    assert _close(g, fd, 1e-4) < 1e-4


@pytest.mark.gpu
def test_gpu_adjoint_matches_oracle(sty, cuda):
    import torch
    import ctypes as C
    W, H, S, R = 48, 32, 4, 6
    planes, valid, rec, p, pt = _case(sty, W, H, S, seed=9)
    target = _target(oracle, rec, pt, R, W, H)
    loss_ref, g_ref = oracle.pf_adjoint(rec, 0, R, p, 8, target)
    fd = _fd(oracle, rec, p, R, target)
    assert _close(g_ref, fd, 1e-4) < 1e-4
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, 1)
    tg = torch.from_numpy(target.astype(np.float32)).cuda()
    grad = torch.zeros(36, dtype=torch.float32, device="cuda")
    prm = (C.c_float * 36)(*p.astype(np.float32))
    loss = C.c_float()
    sty.check(sty.lib().sty_pf_adjoint(C.byref(rs.c()), 0, R, prm, 8, None, tg.data_ptr(), grad.data_ptr(),
                                       C.byref(loss), None))
    torch.cuda.synchronize()
    g = grad.cpu().numpy().astype(np.float64)
    assert abs(loss.value - loss_ref) <= 1e-4 * loss_ref
    assert _close(g, g_ref, 1e-4) < 1e-4, f"vs analytic {_close(g, g_ref, 1e-4):.2e}"
    assert _close(g, fd, 1e-4) < 1e-4, f"vs FD {_close(g, fd, 1e-4):.2e}"


def _bench_params(rng, bandwidths):
    """The adjoint workload's parameter vector: sharpness 50, 8 sorted thresholds, 8 sorted RGB
    ramp colours, the three filter bandwidths."""
    p = np.zeros(36)
    p[0] = 50.0
    p[1:9] = np.sort(rng.uniform(0.05, 1.2, 8))
    p[9:33] = np.sort(rng.uniform(0.0, 1.0, 24))
    p[33:36] = bandwidths
    return p


def _perturbed(p, seed=1):
    """The target's parameter vector: p perturbed by Gaussian noise of sigma 0.05 (relative), seed 1."""
    pt = p + np.random.default_rng(seed).normal(0.0, 0.05, 36) * np.abs(p)
    pt[33:36] = np.abs(pt[33:36])
    return pt


def _gpu_adjoint(sty, rs, R, p, target, in_next_dev=None, fn="sty_pf_adjoint"):
    import ctypes as C
    import torch
    tg = torch.from_numpy(np.ascontiguousarray(target, dtype=np.float32)).cuda()
    grad = torch.zeros(36, dtype=torch.float32, device="cuda")
    loss = C.c_float()
    sty.check(getattr(sty.lib(), fn)(C.byref(rs.c()), 0, R, (C.c_float * 36)(*p.astype(np.float32)), 8,
                                     None if in_next_dev is None else in_next_dev.data_ptr(), tg.data_ptr(),
                                     grad.data_ptr(), C.byref(loss), None))
    torch.cuda.synchronize()
    return loss.value, grad.cpu().numpy().astype(np.float64)


def _fd_in(orc, rec, p, R, target, in_next):
    """FP64 central differences with a step of 1e-4 relative to each parameter (1e-4 where it is 0):
    an absolute 1e-4 is 2e-3 of a position bandwidth of 0.05, whose weights exp(-d^2 / 2 sigma^2)
    then bend enough within the step to leave a truncation error above 1e-4."""
    g = np.zeros(36)
    for k in range(36):
        h = H_FD * abs(p[k]) if p[k] != 0 else H_FD
        e = np.zeros(36)
        e[k] = h
        g[k] = (orc.pf_adjoint_loss(rec, 0, R, p + e, 8, target, in_next) -
                orc.pf_adjoint_loss(rec, 0, R, p - e, 8, target, in_next)) / (2 * h)
    return g


@pytest.mark.gpu
def test_gpu_adjoint_benchmark_shape_matches_fd(sty, cuda):
    """The benchmarked shape: radius 16, 4 spp, sharpness 50, bandwidths (8, 0.5, 0.2), a child
    input, on records with the filter workload's per-tile spread (every tile of the forward filter
    takes the expanded exponent form the benchmark runs): all 36 gradient entries against FP64
    central differences (step 1e-4 relative) and the FP64 analytic adjoint, within 1e-4 relative."""
    import torch
    import bench
    W, H, S, R = 64, 48, 4, 16
    planes, valid = sty.synth.records(W, H, S, 1, seed=31, offset_scale=0.2)
    assert bench.expanded_fraction(planes, valid, W, H, S, 1, 0.5) == 1.0
    rec = sty.pf.host_records(planes, valid, W, H, S, 1)
    rng = np.random.default_rng(31)
    p = _bench_params(rng, [8.0, 0.5, 0.2])
    child = rng.random((3, W * H * S)).astype(np.float32)
    target = oracle.pf_adjoint_image(rec, 0, R, _perturbed(p), 8, child.astype(np.float64))
    loss_ref, g_ref = oracle.pf_adjoint(rec, 0, R, p, 8, target, child.astype(np.float64))
    fd = _fd_in(oracle, rec, p, R, target, child.astype(np.float64))
    assert _close(g_ref, fd, 1e-4) < 1e-4
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, 1)
    loss, g = _gpu_adjoint(sty, rs, R, p, target, torch.from_numpy(child).cuda())
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    assert _close(g, g_ref, 1e-4) < 1e-4, f"vs analytic {_close(g, g_ref, 1e-4):.2e}"
    assert _close(g, fd, 1e-4) < 1e-4, f"vs FD {_close(g, fd, 1e-4):.2e}"


@pytest.mark.gpu
def test_gpu_adjoint_on_traced_records_matches_fd(sty, cuda):
    """The adjoint on the traced Cornell-box records (the plain NL-PF workload's buffers, 4 paths per
    pixel): depth 0 with the filtered depth-1 result as its child input, radius 8, bandwidths
    (4, 0.05, 0.2), target rendered from the parameters perturbed by N(0, 0.05^2) (seed 1); all 36
    entries against FP64 central differences (step 1e-4 relative) and the analytic adjoint within
    1e-4 relative."""
    import torch
    a = sty.abi
    W, H, S, R = 64, 48, 4, 8
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    cfg = sty.scene.screen_render_config(max_depth=2, branch=S, radius=R, sigma_pixel=0.0, sigma_pos=0.05,
                                         sigma_nrm=0.2, screen_style=0, seed=0)
    style = a.style_program([a.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0], depth_mask=1 << 1)])
    rs3, _, _ = sc.trace_records(cfg, [style])
    out = sty.pf_screen_filter(rs3, sty.ScreenParams(R, 0.0, 0.05, 0.2), style)
    torch.cuda.synchronize()
    n = W * H * S
    planes = rs3.planes[:, :n].contiguous().cpu().numpy()  # depth 0
    valid = rs3.valid[:n].contiguous().cpu().numpy()
    child = out[1].contiguous()
    childh = child.cpu().numpy().astype(np.float64)
    rec = sty.pf.host_records(planes, valid, W, H, S, 1)
    rng = np.random.default_rng(7)
    p = _bench_params(rng, [4.0, 0.05, 0.2])
    p[1:9] = np.sort(rng.uniform(0.02, 0.8, 8))  # thresholds across the render's luminance range
    target = oracle.pf_adjoint_image(rec, 0, R, _perturbed(p), 8, childh)
    loss_ref, g_ref = oracle.pf_adjoint(rec, 0, R, p, 8, target, childh)
    fd = _fd_in(oracle, rec, p, R, target, childh)
    assert _close(g_ref, fd, 1e-4) < 1e-4
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, 1)
    loss, g = _gpu_adjoint(sty, rs, R, p, target, child)
    assert loss_ref > 0 and abs(loss - loss_ref) <= 1e-4 * loss_ref
    assert _close(g, g_ref, 1e-4) < 1e-4, f"vs analytic {_close(g, g_ref, 1e-4):.2e}"
    assert _close(g, fd, 1e-4) < 1e-4, f"vs FD {_close(g, fd, 1e-4):.2e}"
    sc.close()
