"""Multi-GPU path on the CPU: two ranks over gloo run the replica logic the bench uses
(per-rank source shards, max of the ranks' timed intervals, whole-job rate)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "c-2graph_gb300"))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, vlist, out):
    import torch.distributed as dist

    sys.path.insert(0, os.path.join(ROOT, "c-2graph_gb300"))
    from c2g import replicas

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        src = replicas.rank_sources(vlist, 64, rank, 2024)
        local_ms = 100.0 + 50.0 * rank  # rank 1 is the slower one
        slowest = replicas.max_over_ranks(local_ms)
        out.put((rank, src.tolist(), slowest, replicas.job_rate(64 * 5, world, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from c2g import replicas

    rng = np.random.default_rng(3)
    deg = rng.integers(0, 40, size=4096)
    vlist = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, vlist, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, m0, j0), (r1, s1, m1, j1) = res
    assert (r0, r1) == (0, 1)
    # both ranks see the slowest rank's time, and the same whole-job rate
    assert m0 == m1 == 150.0
    assert j0 == j1 == pytest.approx(64 * 5 * 2 / 0.150)
    # the shards are distinct draws with the batched configuration's shape
    assert s0 != s1 and len(s0) == len(s1) == 64
    assert s0 == replicas.rank_sources(vlist, 64, 0, 2024).tolist()
    d = np.diff(vlist)
    assert all(d[v] > 0 for v in s0 + s1)
    # without a process group the helpers are the single-GPU identities
    assert replicas.max_over_ranks(7.5) == 7.5


def test_bench_selection_equals_library_rule():
    """bench.py restates the batched configuration's source selection so that its
    reference arm needs nothing from the library; both give the same sources."""
    import bench
    from c2g import replicas

    rng = np.random.default_rng(0)
    for V in (50, 1000, 4096):
        deg = rng.integers(0, 30, size=V)
        deg[rng.choice(V, V // 5, replace=False)] = 0
        vlist = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
        for n, seed in ((256, 2024), (64, 2025), (7, 3)):
            assert np.array_equal(bench.workload_sources(vlist, n, seed), replicas.pick_sources(vlist, n, seed))
