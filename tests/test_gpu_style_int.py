"""GPU checks of the style nodes (vs the FP64 oracle) and of the integer helpers (bit-exact vs
the golden vectors and the oracle)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _gpu_style(sty, prog, depth, rgb):
    import torch
    x = torch.from_numpy(np.ascontiguousarray(rgb, dtype=np.float32)).cuda()
    y = torch.empty_like(x)
    sty.check(sty.lib().sty_style_apply(C.byref(prog), depth, x.data_ptr(), y.data_ptr(), x.shape[0],
                                        torch.cuda.current_stream().cuda_stream or None))
    torch.cuda.synchronize()
    return y.cpu().numpy()


NODES = {
    "toon": lambda a: [a.toon(0.2)],
    "palette": lambda a: [a.palette([(0.1, 0.1, 0.1), (0.8, 0.2, 0.1), (0.2, 0.7, 0.3), (0.9, 0.9, 0.8)], 1.5, 0.5)],
    "sat_adjust": lambda a: [a.sat_adjust(0.6, 1.2)],
    "sat_rex": lambda a: [a.sat_rex(0.3)],
    "eight_bit": lambda a: [a.eight_bit(1.5)],
    "toon_steps": lambda a: [a.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0])],
    "ramp_smooth": lambda a: [a.ramp_smooth(50.0, [0.1, 0.3, 0.6], [(0.1, 0.05, 0.2), (0.5, 0.4, 0.3), (1, .95, .8)])],
    "chain": lambda a: [a.sat_rex(0.4), a.toon(0.25, depth_mask=0b10)],
}


@pytest.mark.parametrize("name", sorted(NODES))
@pytest.mark.parametrize("depth", [0, 1, 3])
def test_style_nodes_match_oracle(sty, orc, cuda, name, depth):
    prog = sty.abi.style_program(NODES[name](sty.abi))
    rng = np.random.default_rng(sum(map(ord, name)) * 10 + depth)
    rgb = np.exp(rng.normal(-1.0, 1.5, size=(20000, 3))).astype(np.float32)
    rgb[:10] = 0.0
    got = _gpu_style(sty, prog, depth, rgb)
    ref = orc.style_apply(prog, depth, rgb.astype(np.float64))
    err = rel_err(got, ref, 1e-6).max(axis=1)
    # quantising nodes may land in the neighbouring band when the input is within float32
    # rounding of a band edge: allow a handful of such records, everything else at 1e-5
    bad = err > 1e-5
    assert bad.sum() <= 20000 * 2e-4, f"{bad.sum()} records off (max {err.max():.3e})"


def test_pcg32_bit_exact(sty, cuda, golden, orc):
    import torch
    streams = golden["pcg32"]["streams"]
    for s in streams:
        seeds = torch.from_numpy(np.array([s["seed"]], dtype=np.uint64)).cuda()
        out = torch.zeros(len(s["draws"]), dtype=torch.uint32, device="cuda")
        st = torch.zeros(2, dtype=torch.uint64, device="cuda")
        sty.check(sty.lib().sty_pcg32_streams(seeds.data_ptr(), s["seq"], 1, len(s["draws"]), out.data_ptr(),
                                              st.data_ptr(), None))
        torch.cuda.synchronize()
        assert out.cpu().numpy().tolist() == s["draws"]
        assert st.cpu().numpy().tolist() == s["state"]
    # many streams vs the oracle
    rng = np.random.default_rng(0)
    seeds = rng.integers(0, 2**63, size=100000, dtype=np.uint64)
    ref, ref_st = orc.pcg32_streams(seeds, 12345, 5)
    sd = torch.from_numpy(seeds).cuda()
    out = torch.zeros((seeds.size, 5), dtype=torch.uint32, device="cuda")
    st = torch.zeros((seeds.size, 2), dtype=torch.uint64, device="cuda")
    sty.check(sty.lib().sty_pcg32_streams(sd.data_ptr(), 12345, seeds.size, 5, out.data_ptr(), st.data_ptr(), None))
    torch.cuda.synchronize()
    assert (out.cpu().numpy() == ref).all()
    assert (st.cpu().numpy() == ref_st).all()


def test_hash_cells_bit_exact(sty, cuda, golden, orc):
    import torch
    h = golden["hash"]

    def run(points, pmin, pmax, res, table):
        p = torch.from_numpy(np.ascontiguousarray(points, dtype=np.float32)).cuda()
        n = p.numel() // 3
        cells = torch.zeros((n, 3), dtype=torch.int32, device="cuda")
        idx = torch.zeros(n, dtype=torch.int32, device="cuda")
        sty.check(sty.lib().sty_hash_cells(p.data_ptr(), n, (C.c_float * 3)(*pmin), (C.c_float * 3)(*pmax),
                                           (C.c_uint32 * 3)(*res), table, cells.data_ptr(), idx.data_ptr(), None))
        torch.cuda.synchronize()
        return cells.cpu().numpy().view(np.uint32), idx.cpu().numpy().view(np.uint32)

    cells, idx = run(np.array(h["points"]), h["pmin"], h["pmax"], h["res"], h["table"])
    assert cells.tolist() == h["cells"] and idx.tolist() == h["index"]
    rng = np.random.default_rng(1)
    pts = rng.uniform(-3, 3, size=(200000, 3)).astype(np.float32)
    args = ([-2.5, -2.0, -3.0], [2.0, 2.5, 3.0], [97, 131, 61], (1 << 26) - 5)
    c_ref, i_ref = orc.hash_cells(pts, *args)
    c_got, i_got = run(pts, *args)
    assert (c_got == c_ref).all() and (i_got == i_ref).all()
