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
