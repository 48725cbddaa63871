"""Replica renders across ranks (one process per GPU).

Neither integrator shards a frame: NL-PF neighbourhoods reach across arbitrary pixels (the world-space
grid) and NL-NRC trains one cache online from the whole image, so a render splits across GPUs only
as replicas, each rendering its own share of the repeats; their FP64 films are combined once at the
end, weighted by the number of repeats each rendered (the reference accumulates every repeat into
one film with the same weight, film.rs:30-50). With the branching path tracer a replica renders
repeats [first, first + count) of one seed's sample sequence, so the combined film equals the
single-process film up to the order of the FP64 additions.

The collective is one all-reduce of the film (and of the timing maximum) through torch.distributed;
no collective runs inside a render.
"""
from __future__ import annotations

import torch


def shard_repeats(total: int, world: int, rank: int) -> tuple[int, int]:
    """(first, count) of the repeats rank `rank` of `world` renders: contiguous, the first
    total % world ranks take one more."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("shard_repeats wants world >= 1, 0 <= rank < world, total >= 0")
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def replica_seed(seed: int, rank: int) -> int:
    """Seed of replica `rank` for integrators whose samples key on the seed alone (NL-PF, NL-NRC):
    splitmix64 of seed + rank, so replicas draw independent streams and rank 0 keeps a fixed
    function of the seed."""
    z = (seed + 0x9E3779B97F4A7C15 * (rank + 1)) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def merge_film(film: torch.Tensor, count: int, group=None) -> torch.Tensor:
    """The repeat-weighted mean of every rank's film (each the mean over its own `count` repeats),
    returned on every rank. FP64; one all-reduce of film * count and one of the counts. A rank with
    no repeats (count 0, more ranks than repeats) renders nothing: its film is not read (it adds
    zeros, so an unset film holding NaN cannot poison the merge). Without an initialised process
    group the film is returned as it is."""
    if film.dtype != torch.float64:
        raise TypeError("merge_film wants the FP64 film")
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return film.clone()
    acc = film * float(count) if count > 0 else torch.zeros_like(film)
    n = torch.tensor([float(count)], dtype=torch.float64, device=film.device)
    torch.distributed.all_reduce(acc, group=group)
    torch.distributed.all_reduce(n, group=group)
    if n.item() <= 0:
        raise ValueError("merge_film: no repeats on any rank")
    return acc / n


def max_over_ranks(x: float, device=None, group=None) -> float:
    """The maximum of a host scalar over the ranks (the job's time is its slowest rank's)."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX, group=group)
    return float(t.item())
