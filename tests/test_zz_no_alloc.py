"""The allocation-free adjoint entry point (sty_pf_adjoint_noalloc).

It exists for callers that cannot allocate device memory: its scratch is one fixed device array
instead of per-call allocations. This file runs last so a failure here never hides the rest of the
suite. The entry point is called through the C ABI twice in a row (the second call finds the
previous call's contents in the shared array) and must agree with sty_pf_adjoint, which allocates
its scratch per call, within the adjoint tests' tolerance (1e-4 relative)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(36, dtype=np.float32)
    p[0] = 5.0
    p[1:9] = np.sort(rng.uniform(0.05, 1.2, 8))
    p[9:33] = np.sort(rng.uniform(0.0, 1.0, 24))
    p[33:36] = [3.0, 0.6, 0.3]
    return p


def _run(sty, fn, rs, R, p, target):
    import torch
    grad = torch.full((36,), float("nan"), dtype=torch.float32, device="cuda")
    loss = C.c_float()
    sty.check(fn(C.byref(rs.c()), 0, R, (C.c_float * 36)(*p), 8, None, target.data_ptr(), grad.data_ptr(),
                 C.byref(loss), None))
    torch.cuda.synchronize()
    return grad.cpu().numpy().astype(np.float64), loss.value


def _rel(a, b):
    scale = np.maximum(np.abs(b), 1e-3 * np.abs(b).max())
    return (np.abs(a - b) / scale).max()


def test_noalloc_adjoint_matches_allocating_entry_point(sty, cuda):
    import torch
    lib = sty.lib()
    results = []
    # two different problems back to back, each checked against the allocating entry point
    for W, H, S, R, seed in ((64, 40, 4, 6, 3), (96, 64, 4, 8, 4)):
        planes, valid = sty.synth.records(W, H, S, 1, seed=seed)
        rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, 1)
        target = torch.rand((W * H * 3,), generator=torch.Generator(device="cuda").manual_seed(seed),
                            device="cuda")
        p = _params(seed)
        g_ref, l_ref = _run(sty, lib.sty_pf_adjoint, rs, R, p, target)
        g_na, l_na = _run(sty, lib.sty_pf_adjoint_noalloc, rs, R, p, target)
        assert np.isfinite(g_na).all()
        assert _rel(g_na, g_ref) < TOL
        assert abs(l_na - l_ref) <= TOL * abs(l_ref)
        results.append((g_na, l_na))
    assert not np.allclose(results[0][0], results[1][0])  # the second call computed its own answer


def test_noalloc_adjoint_allocates_no_device_memory(sty, cuda):
    """The property the entry point exists for: after a first call on the device (which looks up the
    scratch array's address and loads the kernels), further calls leave the device's free memory
    exactly unchanged."""
    import torch
    lib = sty.lib()
    W, H, S, R = 80, 48, 4, 6
    planes, valid = sty.synth.records(W, H, S, 1, seed=8)
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, 1)
    target = torch.rand((W * H * 3,), generator=torch.Generator(device="cuda").manual_seed(8), device="cuda")
    p = _params(8)
    _run(sty, lib.sty_pf_adjoint_noalloc, rs, R, p, target)  # first call on the device: set-up
    grad = torch.zeros(36, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        sty.check(lib.sty_pf_adjoint_noalloc(C.byref(rs.c()), 0, R, (C.c_float * 36)(*p), 8, None,
                                             target.data_ptr(), grad.data_ptr(), None, None))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.isfinite(grad).all()


def test_noalloc_adjoint_rejects_oversize_input(sty, cuda):
    import torch
    lib = sty.lib()
    W, H, S = 512, 160, 4  # 327,680 records per depth > 2^18
    planes, valid = sty.synth.records(W, H, S, 1, seed=1)
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, 1)
    target = torch.zeros(W * H * 3, device="cuda")
    grad = torch.zeros(36, device="cuda")
    st = lib.sty_pf_adjoint_noalloc(C.byref(rs.c()), 0, 4, (C.c_float * 36)(*_params(0)), 8, None,
                                    target.data_ptr(), grad.data_ptr(), None, None)
    assert st == sty.STY_ERR_ARG
    assert b"fixed scratch limit" in lib.sty_last_error()
