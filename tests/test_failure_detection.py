"""Failure detection without a GPU fault: every spin-wait in the library is bounded and, when it
gives up, ORs STY_DEV_WAIT_TIMEOUT into the device status word and returns. The probe kernel waits
on an mbarrier that nothing completes (the timeout path in isolation); the context must stay
usable afterwards. Argument errors are reported without touching the GPU."""
import time

import numpy as np
import pytest


def test_probe_rejects_bad_limits(sty):
    for bad in (0, 2000001):
        assert sty.lib().sty_wait_timeout_probe(bad, None) == sty.STY_ERR_ARG


@pytest.mark.gpu
def test_bounded_wait_times_out_and_context_survives(sty, cuda):
    import torch
    assert sty.abi.device_status() == 0
    t0 = time.perf_counter()
    sty.check(sty.lib().sty_wait_timeout_probe(20000, None))  # 20 ms
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert sty.abi.device_status() == sty.abi.STY_DEV_WAIT_TIMEOUT  # read and cleared
    assert sty.abi.device_status() == 0
    assert 0.015 <= dt < 5.0, dt
    # the context still runs the filter and matches a second, clean run
    W, H, S, D = 48, 24, 4, 1
    planes, valid = sty.synth.records(W, H, S, D, seed=3)
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, D)
    prm = sty.ScreenParams(radius=4, sigma_pixel=2.0, sigma_pos=0.5, sigma_nrm=0.2)
    a = sty.pf_screen_filter(rs, prm, None).clone()
    b = sty.pf_screen_filter(rs, prm, None)
    torch.cuda.synchronize()
    assert torch.equal(a, b) and bool(torch.isfinite(a).all())
    assert np.abs(a.cpu().numpy()).max() > 0
    assert sty.abi.device_status() == 0
