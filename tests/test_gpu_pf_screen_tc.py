"""GPU parity of the tcgen05 screen filter (STY_SCREEN_KERNEL_TENSOR: 4 spp, radius 15 or 16) against
the FP64 oracle, through the C ABI.

Tolerance: as for the CUDA-core kernels, filtered radiance within 1e-5 relative of the FP64 oracle
on the same buffers; styled outputs at the same tolerance except where the oracle's filtered
luminance sits within 1e-5 (relative) of a hard toon threshold."""
import numpy as np
import pytest

from conftest import rel_err
from test_gpu_pf_screen import TOL, _depth_parity, _setup

pytestmark = pytest.mark.gpu


@pytest.fixture
def tensor_kernel(sty):
    sty.set_screen_kernel(sty.SCREEN_KERNEL_TENSOR)
    yield
    sty.set_screen_kernel(sty.SCREEN_KERNEL_AUTO)


@pytest.mark.parametrize("R", [15, 16])
@pytest.mark.parametrize("sigma_pos", [0.5, 0.2])
def test_tc_filter_depth_matches_oracle(sty, orc, cuda, tensor_kernel, R, sigma_pos):
    """Ragged image (not a multiple of the 8x4 tile); sigma_pos 0.2 spreads the scaled positions of
    many tiles beyond the bilinear form's bound, so those tiles take the direct form."""
    W, H, S, D = 70, 37, 4, 1
    planes, valid, rs, hrec = _setup(sty, W, H, S, D, seed=400 + R)
    prm = sty.ScreenParams(radius=R, sigma_pixel=R / 2, sigma_pos=sigma_pos, sigma_nrm=0.2)
    _, got_o, ref_o, _, m, ef = _depth_parity(sty, orc, rs, hrec, valid, 0, prm, None)
    assert ef < TOL, f"filtered rel err {ef:.3e}"
    assert rel_err(got_o[:, m], ref_o[:, m], 1e-6).max() < TOL


def test_tc_image_smaller_than_a_tile(sty, orc, cuda, tensor_kernel):
    """A 6 x 3 image: one partial tile, every candidate row and column partly outside the image."""
    W, H, S, D = 6, 3, 4, 1
    planes, valid, rs, hrec = _setup(sty, W, H, S, D, seed=91)
    prm = sty.ScreenParams(radius=16, sigma_pixel=8.0, sigma_pos=0.5, sigma_nrm=0.2)
    _, got_o, ref_o, _, m, ef = _depth_parity(sty, orc, rs, hrec, valid, 0, prm, None)
    assert ef < TOL, f"filtered rel err {ef:.3e}"


def test_tc_unaligned_planes_take_the_cuda_core_kernel(sty, cuda, tensor_kernel):
    """Record planes off the 16-byte boundary cannot be bulk-copied: the call must give exactly the
    CUDA-core kernel's result."""
    import torch
    W, H, S, D = 40, 24, 4, 1
    planes, valid = sty.synth.records(W, H, S, D, seed=92)
    n = W * H * S
    big = torch.zeros((12, n + 1), dtype=torch.float32, device="cuda")
    big[:, 1:] = torch.from_numpy(planes).cuda()
    rs = sty.RecordSet(big[:, 1:], torch.from_numpy(valid).cuda(), W, H, S, D)  # planes 4 bytes past a boundary
    prm = sty.ScreenParams(radius=16, sigma_pixel=8.0, sigma_pos=0.5, sigma_nrm=0.2)
    got = sty.pf_screen_filter_depth(rs, 0, prm, None)
    sty.set_screen_kernel(sty.SCREEN_KERNEL_FP32)
    ref = sty.pf_screen_filter_depth(rs, 0, prm, None)
    torch.cuda.synchronize()
    assert torch.equal(got, ref)


def test_tc_pixel_term_off_and_tight_records(sty, orc, cuda, tensor_kernel):
    """sigma_pixel <= 0 (no pixel-distance term: the table holds 0 inside the window) on records
    packed close together (offset_scale 0.2)."""
    W, H, S, D = 48, 40, 4, 1
    planes, valid, rs, hrec = _setup(sty, W, H, S, D, seed=77, offset_scale=0.2)
    prm = sty.ScreenParams(radius=16, sigma_pixel=0.0, sigma_pos=0.5, sigma_nrm=0.2)
    _, got_o, ref_o, _, m, ef = _depth_parity(sty, orc, rs, hrec, valid, 0, prm, None)
    assert ef < TOL, f"filtered rel err {ef:.3e}"


def test_tc_full_chain_c2_style(sty, orc, cuda, tensor_kernel):
    """All depths with the C2 toon node at depth 1, each depth against the oracle run on the GPU's
    own deeper-depth output."""
    import torch
    W, H, S, D = 96, 64, 4, 5
    planes, valid, rs, hrec = _setup(sty, W, H, S, D, seed=0)
    prm, style = sty.c2_params(), sty.c2_style()
    out_all = sty.pf_screen_filter(rs, prm, style)
    torch.cuda.synchronize()
    thresholds = np.array([0.1, 0.3, 0.6], dtype=np.float32).astype(np.float64)
    for d in range(D - 1, -1, -1):
        nxt = out_all[d + 1] if d + 1 < D else None
        _, got_o, ref_o, ref_f, m, ef = _depth_parity(sty, orc, rs, hrec, valid, d, prm, style, nxt)
        assert ef < TOL, f"depth {d}: filtered rel err {ef:.3e}"
        near = np.zeros(m.size, dtype=bool)
        if d == 1:
            lum = ref_f[0] * 0.2126 + ref_f[1] * 0.7152 + ref_f[2] * 0.0722
            for t in thresholds:
                near |= np.abs(lum - t) <= 1e-5 * t
        keep = m & ~near
        assert rel_err(got_o[:, keep], ref_o[:, keep], 1e-6).max() < TOL


def test_tc_c2_full_size_sampled_parity(sty, orc, cuda, tensor_kernel):
    """The benchmark workload at full size (1920x1080 x 4 spp x 5 depths, radius 16, toon at depth 1)
    on the tensor-core kernel: 1500 sampled records per depth against the FP64 oracle, and every
    record within 2e-5 of the CUDA-core kernel's output."""
    import torch
    W, H, S, D = 1920, 1080, 4, 5
    planes, valid = sty.synth.records(W, H, S, D, seed=0)
    rs = sty.RecordSet.from_numpy(planes, valid, W, H, S, D)
    hrec = sty.pf.host_records(planes, valid, W, H, S, D)
    prm, style = sty.c2_params(), sty.c2_style()
    out_all = sty.pf_screen_filter(rs, prm, style)
    torch.cuda.synchronize()
    n = rs.n_per_depth
    rng = np.random.default_rng(7)
    thresholds = np.array([0.1, 0.3, 0.6], dtype=np.float32).astype(np.float64)
    for d in range(D - 1, -1, -1):
        idx = np.sort(rng.choice(n, size=1500, replace=False))
        nxt = out_all[d + 1].cpu().numpy().astype(np.float64) if d + 1 < D else None
        ref_o, ref_f = orc.pf_screen_filter_records(hrec, d, prm.c(), style, idx, out_next=nxt)
        got = out_all[d][:, torch.from_numpy(idx.astype(np.int64)).cuda()].cpu().numpy()
        m = valid[d * n + idx].astype(bool)
        assert (got[:, ~m] == 0).all()
        near = np.zeros(idx.size, dtype=bool)
        if d == 1:
            lum = ref_f[0] * 0.2126 + ref_f[1] * 0.7152 + ref_f[2] * 0.0722
            for t in thresholds:
                near |= np.abs(lum - t) <= 1e-5 * t
        keep = m & ~near
        assert keep.sum() > 1200
        err = rel_err(got[:, keep], ref_o[:, keep], 1e-6).max()
        assert err < TOL, f"depth {d}: rel err {err:.3e}"
    # every record of the unstyled deepest depth against the CUDA-core kernel
    filt_tc = torch.empty((3, n), dtype=torch.float32, device="cuda")
    sty.pf_screen_filter_depth(rs, D - 1, prm, None, filtered=filt_tc)
    sty.set_screen_kernel(sty.SCREEN_KERNEL_FP32)
    filt_fp = torch.empty((3, n), dtype=torch.float32, device="cuda")
    sty.pf_screen_filter_depth(rs, D - 1, prm, None, filtered=filt_fp)
    torch.cuda.synchronize()
    mv = torch.from_numpy(valid[(D - 1) * n:D * n].astype(bool)).cuda()
    a, b = filt_tc[:, mv], filt_fp[:, mv]
    diff = ((a - b).abs() / b.abs().clamp_min(1e-6)).max().item()
    assert diff < 2e-5, f"tensor vs CUDA-core kernel: {diff:.3e}"
