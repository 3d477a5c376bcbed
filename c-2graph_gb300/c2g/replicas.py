"""Replica scheduling of the query mix over several GPUs (one process per GPU).

Queries are independent, so N GPUs run N replicas: each rank holds the whole graph,
runs its own share of sources, and the job's rate is the sum of all ranks' queries over
the slowest rank's time.  There is no collective on the data path; the only exchange is
the max of the ranks' timed intervals.  The reference has no multi-GPU path (its PM
mode pairs one GPU with a CPU thread, src/sssp/purn-perk/Main.cu:87-246).
"""
import numpy as np


def pick_sources(vlist, n, seed):
    """The batched configuration's selection: half uniform over vertices with
    out-edges, half from the top 1% out-degree vertices (seeded)."""
    deg = np.diff(vlist)
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(deg > 0)
    top = np.argsort(-deg, kind="stable")[:max(1, len(deg) // 100)]
    top = top[deg[top] > 0]
    half = n // 2
    # small graphs: draw with replacement when a set is smaller than its share
    out = np.concatenate([rng.choice(cand, n - half, replace=len(cand) < n - half),
                          rng.choice(top, half, replace=len(top) < half)])
    return out.astype(np.int32)


def rank_sources(vlist, n, rank, base_seed):
    """Rank `rank`'s share: its own seeded draw of n sources (weak scaling: every rank
    runs a full batch)."""
    return pick_sources(vlist, n, base_seed + rank)


def max_over_ranks(value, device=None):
    """Max of a per-rank float over the default process group (the value itself when
    torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(queries_per_rank, world, slowest_ms):
    """Whole-job queries per second: every rank's queries over the slowest rank's time."""
    return queries_per_rank * world / (slowest_ms / 1000.0)
