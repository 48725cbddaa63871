"""Replica renders over ranks (the only way a render spreads over GPUs: neither integrator shards a
frame). CPU: two gloo ranks on 127.0.0.1 exercise the repeat split, the FP64 film merge and the
timing maximum. GPU: a branching path tracer render split into two replica calls (first_repeat)
merges to the single render's film."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out, total=7):
    import sys
    sys.path.insert(0, os.getcwd())
    import __graft_entry__ as g
    rp = g.package().replicas
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        first, count = rp.shard_repeats(total, world, rank)
        # each rank's film: the mean over its repeats of a per-repeat image f(r) = r + pixel index;
        # a rank without repeats never renders, so its film is left unset (NaN)
        px = torch.arange(6, dtype=torch.float64)
        if count:
            film = torch.stack([r + px for r in range(first, first + count)]).mean(0)
        else:
            film = torch.full((6,), float("nan"), dtype=torch.float64)
        merged = rp.merge_film(film, count)
        t = rp.max_over_ranks(10.0 * (rank + 1))
        out.put((rank, first, count, merged.numpy(), t, rp.replica_seed(5, rank)))
    finally:
        torch.distributed.destroy_process_group()


def test_replicas_merge_over_gloo_ranks(sty):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, f0, c0, m0, t0, s0), (r1, f1, c1, m1, t1, s1) = res
    assert (f0, c0, f1, c1) == (0, 4, 4, 3)  # contiguous, the first rank takes the extra repeat
    want = np.mean([r + np.arange(6) for r in range(7)], axis=0)  # the single-process film
    np.testing.assert_allclose(m0, want, rtol=1e-15)
    np.testing.assert_array_equal(m0, m1)
    assert t0 == t1 == 20.0
    assert s0 != s1


def test_merge_ignores_ranks_without_repeats(sty):
    """One repeat over two ranks: the second rank renders nothing and its unset (NaN) film must not
    reach the merged film."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q, 1)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, f0, c0, m0, _, _), (_, f1, c1, m1, _, _) = res
    assert (f0, c0, c1) == (0, 1, 0)
    np.testing.assert_array_equal(m0, np.arange(6, dtype=np.float64))
    np.testing.assert_array_equal(m0, m1)


def test_shard_repeats_covers_every_repeat(sty):
    rp = sty.replicas
    for total in (0, 1, 5, 64, 1001):
        for world in (1, 2, 3, 8):
            parts = [rp.shard_repeats(total, world, r) for r in range(world)]
            seen = [i for f, c in parts for i in range(f, f + c)]
            assert seen == list(range(total))
            assert max(c for _, c in parts) - min(c for _, c in parts) <= 1
    with pytest.raises(ValueError):
        rp.shard_repeats(4, 2, 2)


def test_merge_film_without_process_group(sty):
    f = torch.arange(4, dtype=torch.float64)
    assert torch.equal(sty.replicas.merge_film(f, 3), f)
    with pytest.raises(TypeError):
        sty.replicas.merge_film(f.float(), 3)
    assert sty.replicas.max_over_ranks(2.5) == 2.5


@pytest.mark.gpu
def test_brpt_replicas_merge_to_the_single_render(sty, cuda):
    """Two replica calls (repeats 0-2 and 3-4 of one seed) weighted by their repeat counts give the
    film of one call rendering repeats 0-4 (FP64 addition order aside)."""
    pos, mids, mats, cam = sty.scene.cornell_box(16, 12, style=(0, -1, -1, -1))
    progs = [sty.abi.style_program([sty.abi.toon(0.2)])]
    sc = sty.scene.Scene(pos, mids, mats, cam)
    cfg = lambda first, n: sty.scene.brpt_config(max_depth=4, inner_samples=(4, 2), repeats=n, seed=9,  # noqa: E731
                                                 first_repeat=first)
    full, _ = sc.brpt_render(cfg(0, 5), progs)
    parts = [(sc.brpt_render(cfg(f, c), progs)[0], c) for f, c in (sty.replicas.shard_repeats(5, 2, r)
                                                                   for r in range(2))]
    merged = sum(f * c for f, c in parts) / 5
    np.testing.assert_allclose(merged.cpu().numpy(), full.cpu().numpy(), rtol=1e-12, atol=1e-15)
    # a replica is not a re-run of the first repeats
    assert not np.allclose(parts[1][0].cpu().numpy(), sc.brpt_render(cfg(0, 2), progs)[0].cpu().numpy())
    sc.close()


def test_oracle_brpt_replicas_merge(sty):
    """The oracle's branching path tracer keys on the same (seed, repeat) as the GPU: two replica
    runs of repeats 0-1 and 2 merge (repeat-weighted) to the single run of repeats 0-2."""
    import oracle
    pos, mids, mats, cam = sty.scene.cornell_box(8, 6, style=(0, -1, -1, -1))
    progs = [sty.abi.style_program([sty.abi.toon(0.2)])]
    marr = (sty.scene.SceneMaterial * len(mats))(*mats)
    camv = list(cam.eye) + list(cam.target) + list(cam.up) + [cam.fov_y, cam.width, cam.height, cam.filter_radius]
    run = lambda first, n: oracle.brpt(pos, mids, marr, camv, progs, 3, (2,), repeats=n, seed=4,  # noqa: E731
                                       first_repeat=first)
    full = run(0, 3)
    merged = (run(0, 2) * 2 + run(2, 1)) / 3
    np.testing.assert_allclose(merged, full, rtol=1e-12, atol=1e-15)
    assert not np.allclose(run(2, 1), run(0, 1))
