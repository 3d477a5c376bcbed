"""Benchmark: queries/s of the C^2graph traversal path on one GB300 (and GTEPS).

Workload (default): the scale-22 R-MAT graph of the single-query / batched
configurations (4,194,304 vertices, edge factor 16, a/b/c/d = 0.57/0.19/0.19/0.05,
seed 2, int32 weights in [1,1000], flist = out-normalised uniform(0,1)), pruned by
this library's purn-sssp / purn-ppr (byte-identical to the reference tools).  The
query mix is the batched configuration's: 256 SSSP + 256 PPR sources, half uniform
over vertices with out-edges, half from the top 1% out-degree vertices (selection
seed 2024).  A step runs the whole mix through the batched path, one persistent
launch per kind:
  SSSP: 256 sources, sssp-purn on sssp/ with each source's own record as seeds (EXACT
        mode), int32 distances (bit-exact against the oracle in tests/);
  PPR:  256 sources, ppr-purn on ppr/ (alpha 0.15, rmax 1e-7, FP32; L1 <= 1e-6 vs the
        FP64 oracle in tests/).
value = queries per second with the graph and outputs resident in HBM (CUDA events on
the stream the kernels run on); e2e = the same through the C ABI with pinned host
output buffers (device->host copy of every result inside the timed region).  The plain
per-query GPU path is timed on a sample of the same sources for the
batched-vs-per-query ratio.  Graph and state are larger than L2, so no flush is needed
between steps.

--impl reference times the reference's CPU implementation of the path (the oracle's
restatement of the reference CPU Bellman-Ford / BSP push, all host threads, one query
per thread) on a bounded sample of the same query mix.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "c-2graph_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "queries/s batched vs per-query (SSSP exact, PPR L1<=1e-6) & GTEPS, 1xGB300"
ALPHA, RMAX = 0.15, 1e-7


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def measured_peak():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [x.strip() for x in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_dataset(tools, d, scale, ef, seed, device=None):
    """The step's inputs in <d>: the R-MAT graph (int32 weights in [1, 1000], flist),
    pruned by purn-sssp and by purn-ppr for the step's alpha (folded edges carry
    1 - alpha).  `tools` is the library (c2g) for our arm and the oracle's restatement for
    the reference arm; both write the same bytes (tests/test_oracle_golden.py).  With a
    device, the library generates and prunes on that GPU (the same bytes again:
    tests/test_gpu_ingest.py, tests/test_gpu_prune.py)."""
    t0 = time.time()
    if device is None:
        tools.rmat_write(d, scale, ef, seed, 1, 1000)
    else:
        tools.rmat_write(d, scale, ef, seed, 1, 1000, gpu=True, device=device)
    t1 = time.time()
    if device is None:
        tools.prune_sssp(d)
        tools.prune_ppr(d, alpha=ALPHA)
    else:
        tools.prune_sssp_device(d, device=device)
        tools.prune_ppr_device(d, ALPHA, device=device)
    return t1 - t0, time.time() - t1


def workload_sources(vlist, n, seed):
    """The batched configuration's selection: half uniform over vertices with out-edges,
    half from the top 1% out-degree vertices (seeded; SSSP seed 2024, PPR 2025, plus the
    rank under torchrun).  The same rule as c2g.replicas.pick_sources, restated here so
    the reference arm needs nothing from the library."""
    deg = np.diff(vlist)
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(deg > 0)
    top = np.argsort(-deg, kind="stable")[:max(1, len(deg) // 100)]
    top = top[deg[top] > 0]
    half = n // 2
    out = np.concatenate([rng.choice(cand, n - half, replace=len(cand) < n - half),
                          rng.choice(top, half, replace=len(top) < half)])
    return out.astype(np.int32)


def step_config(args, V, e_sssp, e_ppr, nS, nP, world):
    return {"workload": "rmat-s%d-ef%d pruned, batched multi-tenant mix: %d SSSP + %d PPR sources per step"
                        % (args.scale, args.edge_factor, nS, nP),
            "vertices": V, "edges_sssp": e_sssp, "edges_ppr": e_ppr,
            "sssp": "sssp-purn on sssp/, each source's own record as seeds (EXACT), int32 distances",
            "ppr": "ppr-purn on ppr/ pruned for alpha %.2f, seeded first hop, alpha %.2f, rmax %g" % (ALPHA, ALPHA,
                                                                                                  RMAX),
            "alpha": ALPHA, "rmax": RMAX,
            "sources": "half uniform over vertices with out-edges, half from the top 1% out-degree",
            "l2": "graph and state larger than L2 (no flush needed)",
            "parallelism": "replicas (query-sharded)" if world > 1 else "single GPU"}


def step_ppr_params(g):
    """The step's PPR parameters: alpha 0.15, rmax 1e-7, seeded first hop (ppr-purn),
    the reference's 500-round cap."""
    return g.ppr_params(alpha=ALPHA, rmax=RMAX, seeded=1, max_iter=500)


def cpu_queries(s_ds, p_ds, ssrc, psrc, threads):
    """The reference's CPU implementation of the step's queries (oracle restatement):
    the reference CPU Bellman-Ford from each SSSP source and its record seeds on sssp/,
    and the BSP push in FP32 from each PPR source's first hop on ppr/; one query per
    host thread.  s_ds / p_ds are the sssp/ and ppr/ arrays (oracle.load_dataset).
    Returns the elapsed seconds."""
    import oracle

    ss, ps = oracle.query_seeds(s_ds, ssrc, "sssp"), oracle.query_seeds(p_ds, psrc, "ppr")
    t0 = time.time()
    oracle.batch("sssp", s_ds["vlist"], s_ds["elist"], s_ds["wlist"], None, ssrc, threads=threads, seeds=ss)
    oracle.batch("ppr", p_ds["vlist"], p_ds["elist"], None, p_ds["wlist"], psrc, alpha=ALPHA, rmax=RMAX,
                 max_iter=500, threads=threads, seeds=ps)
    return time.time() - t0


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU implementation of the path (the oracle's
    restatement of its CPU Bellman-Ford and of the push), all host threads, one query
    per thread and kind, on the same inputs and sources as our arm.  Inputs are written
    by the oracle's own R-MAT writer and pruners; nothing here loads the library."""
    if rank != 0:
        return
    import oracle

    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory(dir=args.workdir) as d:
        make_dataset(oracle, d, args.scale, args.edge_factor, args.seed)
        s_ds, p_ds = oracle.load_dataset(d, "sssp"), oracle.load_dataset(d, "ppr")
        svl, pvl = s_ds["vlist"], p_ds["vlist"]
        V = len(svl) - 1
        nS, nP = args.sssp_per_step, args.ppr_per_step
        ssrc = workload_sources(svl, nS, 2024)
        psrc = workload_sources(pvl, nP, 2025)
        # a bounded sample per step: one query per host thread and kind, rotating
        # through the step's sources
        ns = min(threads, nS)
        npq = min(threads, nP)
        times, q_total = [], 0
        for step in range(args.warmup + args.steps):
            dt = cpu_queries(s_ds, p_ds, np.roll(ssrc, -(step * ns) % nS)[:ns], np.roll(psrc, -(step * npq) % nP)[:npq],
                             threads)
            if step >= args.warmup:
                times.append(dt)
                q_total += ns + npq
        cfg = step_config(args, V, int(svl[-1]), int(pvl[-1]), nS, nP, world)
    v = q_total / sum(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "queries/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 (SSSP) + f32 (PPR)", "data": "synthetic R-MAT (seeded); no public dataset",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": "%d SSSP + %d PPR queries of the step's sources per step, one per host "
                                       "thread" % (ns, npq)},
            "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    import c2g

    dev = local_rank
    torch.cuda.set_device(dev)
    dist_on = world > 1
    if dist_on:
        import torch.distributed as tdist

        tdist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    work = tempfile.mkdtemp(dir=args.workdir)
    gen_s, prune_s = make_dataset(c2g, work, args.scale, args.edge_factor, args.seed, device=dev)
    so = {"vlist": c2g.read_array(os.path.join(work, "sssp", "vlist.bin"))}
    po = {"vlist": c2g.read_array(os.path.join(work, "ppr", "vlist.bin"))}
    V = len(so["vlist"]) - 1
    nS, nP = args.sssp_per_step, args.ppr_per_step
    from c2g import replicas

    # every rank runs a full batch of its own draw (weak scaling)
    ssrc = workload_sources(so["vlist"], nS, 2024 + rank)
    psrc = workload_sources(po["vlist"], nP, 2025 + rank)

    gs = c2g.Graph.load(work, "sssp", device=dev)
    gp = c2g.Graph.load(work, "ppr", device=dev)
    stream = torch.cuda.Stream(device=dev)
    gs.set_stream(stream.cuda_stream)
    gp.set_stream(stream.cuda_stream)
    gs.sssp_config(delta=args.delta, tile=args.tile)
    prm = step_ppr_params(gp)
    # Round shape of the batched push from the project's autotuner, on this step's batch
    # (outside the timed region).
    pull_ratio = gp.ppr_batch_autotune(psrc, prm, reps=1)
    big, mn = gs.sssp_batch_autotune(ssrc, seeds=True, mode=c2g.SEEDS_EXACT, reps=1)
    sssp_tile = {"big_steps": big, "min_tiles_per_warp": mn,
                 "rule": "rounds with >= min_tiles_per_warp big tiles per warp walk big tiles, else 128 steps",
                 "pull_frac": gs.sssp_batch_pull_frac(),
                 "pull_rule": "rounds with more than pull_frac * E * Q (query, edge) relaxations pull over the "
                              "reverse CSR"}
    dist_d = torch.empty((nS, V), dtype=torch.int32, device=dev)
    pr_d = torch.empty((nP, V), dtype=torch.float32, device=dev)
    dist_h = torch.empty((nS, V), dtype=torch.int32).pin_memory().numpy()
    pr_h = torch.empty((nP, V), dtype=torch.float32).pin_memory().numpy()

    def step(host):
        """One step: the whole query mix, each kind in one batched launch."""
        if host:
            _, ss = gs.sssp_batch(ssrc, seeds=True, mode=c2g.SEEDS_EXACT, out=dist_h)
            _, _, sp = _ppr_into(gp, psrc, prm, pr_h)
        else:
            _, ss = gs.sssp_batch(ssrc, seeds=True, mode=c2g.SEEDS_EXACT, out_ptr=dist_d.data_ptr())
            _, _, sp = gp.ppr_batch(psrc, prm, pr_ptr=pr_d.data_ptr())
        return ss, sp

    def barrier():
        torch.cuda.synchronize(dev)
        if dist_on:
            tdist.barrier()
        torch.cuda.synchronize(dev)

    def timed(host):
        for _ in range(args.warmup):
            step(host)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        acc = {"s_ms": 0.0, "p_ms": 0.0, "s_bytes": 0.0, "p_bytes": 0.0, "s_rel": 0, "p_push": 0, "s_it": 0,
               "p_it": 0}
        e0.record(stream)
        t0 = time.time()
        for _ in range(args.steps):
            ss, sp = step(host)
            acc["s_ms"] += ss.device_ms
            acc["p_ms"] += sp.device_ms
            acc["s_bytes"] += ss.alg_bytes
            acc["p_bytes"] += sp.alg_bytes
            acc["s_rel"] += ss.edges_relaxed
            acc["p_push"] += sp.edges_relaxed
            acc["s_it"] += ss.iterations
            acc["p_it"] += sp.iterations
        e1.record(stream)
        barrier()
        wall = time.time() - t0
        ms = replicas.max_over_ranks(e0.elapsed_time(e1), device=dev)
        return ms, wall, acc

    with ClockSampler(dev) as clk:
        ms_dev, wall_dev, tot = timed(False)
    ms_e2e, wall_e2e, _ = timed(True)
    q_step = nS + nP
    value = replicas.job_rate(q_step * args.steps, world, ms_dev)
    e2e = replicas.job_rate(q_step * args.steps, world, ms_e2e)

    # The plain per-query GPU path on a sample of the same mix (same kernels' single-
    # query form): the batched-vs-per-query ratio of the metric.
    pq_s = pq_p = pq_sb = pq_pb = 0.0
    for s in ssrc[: args.per_query_sample]:
        _, st = gs.sssp(int(s), seeds=True, mode=c2g.SEEDS_EXACT, out_ptr=dist_d.data_ptr())
        pq_s += st.device_ms
        pq_sb += st.alg_bytes
    for s in psrc[: max(1, args.per_query_sample // 2)]:
        _, _, st = gp.ppr(int(s), prm, pr_ptr=pr_d.data_ptr())
        pq_p += st.device_ms
        pq_pb += st.alg_bytes
    ms_sssp_pq = pq_s / args.per_query_sample
    ms_ppr_pq = pq_p / max(1, args.per_query_sample // 2)
    per_query_qps = q_step / ((nS * ms_sssp_pq + nP * ms_ppr_pq) / 1000.0)

    # Graph500-style TEPS of the batched SSSP: out-edges of reached (vertex, query) pairs.
    d_host = dist_d[: min(8, nS)].cpu().numpy()
    deg = np.diff(so["vlist"])
    reached_edges = sum(int(deg[row != c2g.INF_DIST].sum()) for row in d_host) * nS / len(d_host)
    gteps_batched = reached_edges * args.steps / (tot["s_ms"] / 1000.0) / 1e9

    dominant = "s" if tot["s_ms"] >= tot["p_ms"] else "p"
    peak, peak_kind = measured_peak()
    achieved = tot[dominant + "_bytes"] / (tot[dominant + "_ms"] / 1000.0) / 1e9
    kernel_name = "sssp_batch_persistent" if dominant == "s" else "ppr_batch_persistent"
    # DRAM bytes (read + write) per unit processed (push or relaxation), from an ncu
    # capture of the kernel, scaled to this run's average launch.
    # Full-size step (the autotuners' picks): 2,422 GB per 371.46 G pushes for the PPR
    # launch, 290.4 GB per 61.37 G relaxations for the SSSP launch.
    traffic_per_unit = {"p": 2.422e12 / 371.46e9, "s": 290.4e9 / 61.37e9}[dominant]
    units = tot["p_push"] if dominant == "p" else tot["s_rel"]
    traffic = traffic_per_unit * units / args.steps

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle  # CPU-baseline leg only

        # the same inputs and sources, one query per host thread and kind
        threads = os.cpu_count() or 1
        s_ds, p_ds = oracle.load_dataset(work, "sssp"), oracle.load_dataset(work, "ppr")
        k = min(threads, nS, nP) if args.cpu_sample <= 0 else args.cpu_sample
        dt = cpu_queries(s_ds, p_ds, ssrc[:k], psrc[:k], threads)
        cpu = {"value": 2 * k / dt, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": "%d SSSP (reference CPU Bellman-Ford restated, EXACT seeds on sssp/) + %d PPR (BSP push "
                         "in FP32, seeded on ppr/) queries of the step's sources, one per host thread" % (k, k)}
        del s_ds, p_ds

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 (SSSP); PPR: f64 residual state (res, msg, pushed residual), f32 weights and pr",
            "data": "synthetic R-MAT (seeded); no public dataset",
            "config": dict(step_config(args, V, int(so["vlist"][-1]), int(po["vlist"][-1]), nS, nP, world),
                           path="batched, one persistent launch per kind", ppr_pull_ratio=pull_ratio,
                           sssp_tile_steps=sssp_tile),
            "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": 4 * q_step,
                    "d2h_bytes_per_step": 4 * V * q_step},
            "gpu_launches": 4 * args.steps,
            "roofline": {"bound": "hbm", "kernel": kernel_name, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "traffic_note": "DRAM bytes per launch: an ncu capture's bytes per unit, scaled by units",
                         "byte_model": {"p": "FP64 residual layout: 12 B x V x Q init, 40 B per (vertex, word) "
                                             "entry, 8 B per edge-word step, 8 B per (query, edge) push (FP64 "
                                             "message add), 32 B per touched lane (res and msg read + write)",
                                        "s": "4 B x V x Q init, 40 B per entry, 8 B per edge-word step, 8 B per "
                                             "(query, edge) relaxation"}[dominant]},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "detail": {
                "batched_vs_per_query": value / per_query_qps,
                "per_query_qps": per_query_qps,
                "per_query_sssp_ms": ms_sssp_pq, "per_query_ppr_ms": ms_ppr_pq,
                # single-query relaxation against the HBM roofline (algorithmic bytes / time)
                "per_query_sssp_alg_gbs": pq_sb / (pq_s / 1000.0) / 1e9 if pq_s else None,
                "per_query_sssp_roofline_frac": pq_sb / (pq_s / 1000.0) / 1e9 / peak if pq_s else None,
                "per_query_ppr_alg_gbs": pq_pb / (pq_p / 1000.0) / 1e9 if pq_p else None,
                "per_query_ppr_roofline_frac": pq_pb / (pq_p / 1000.0) / 1e9 / peak if pq_p else None,
                "batched_sssp_ms_per_step": tot["s_ms"] / args.steps,
                "batched_ppr_ms_per_step": tot["p_ms"] / args.steps,
                "sssp_batched_gteps_graph500": gteps_batched,
                "sssp_relaxations_per_s": tot["s_rel"] / (tot["s_ms"] / 1000.0),
                "ppr_pushes_per_s": tot["p_push"] / (tot["p_ms"] / 1000.0),
                "sssp_rounds": tot["s_it"] / args.steps, "ppr_rounds": tot["p_it"] / args.steps,
                "sssp_alg_gbs": tot["s_bytes"] / (tot["s_ms"] / 1000.0) / 1e9,
                "ppr_alg_gbs": tot["p_bytes"] / (tot["p_ms"] / 1000.0) / 1e9,
                "gen_s": gen_s, "prune_s": prune_s, "wall_s_device_run": wall_dev, "wall_s_e2e_run": wall_e2e,
            },
        }
        print(json.dumps(line), flush=True)
    gs.close()
    gp.close()
    if dist_on:
        tdist.destroy_process_group()


def _ppr_into(gp, src, prm, out):
    """Batched PPR with results copied into the caller's (pinned) host array."""
    import ctypes

    import c2g

    st = c2g.Stats()
    s = np.ascontiguousarray(src, dtype=np.int32)
    c2g._check(c2g.lib().c2g_ppr_batch(gp._h, len(s), c2g._ptr(s), ctypes.byref(prm), c2g._ptr(out), None, 0, 0,
                                       ctypes.byref(st)))
    return None, None, st


def run_serve(args):
    """Serving loop (config 5): Poisson arrivals, mix 50% SSSP / 35% PPR / 15% adsorption
    (16 seed labels, per-vertex p_inj/p_cont/p_abnd ~ Dirichlet(1,1,1), 30 iterations) on an
    unpruned R-MAT graph resident in HBM; reports queries/s and p50/p99 latency."""
    import c2g

    rng = np.random.default_rng(7)
    with tempfile.TemporaryDirectory(dir=args.workdir) as d:
        t0 = time.time()
        c2g.rmat_write(d, args.serve_scale, args.edge_factor, 3, 1, 1000)
        gen_s = time.time() - t0
        vl = c2g.read_array(os.path.join(d, "origin", "vlist.bin"))
        V = len(vl) - 1
        cand = np.flatnonzero(np.diff(vl) > 0)
        pp = rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32)
        g = c2g.Graph.load(d, "origin")
        n = args.serve_requests
        kinds = [c2g.REQ_SSSP] * (n * 50 // 100) + [c2g.REQ_PPR] * (n * 35 // 100)
        kinds += [c2g.REQ_ADSORPTION] * (n - len(kinds))
        rng.shuffle(kinds)
        gaps = rng.exponential(1.0 / args.serve_rate, size=n)
        with c2g.Server(g, max_batch=256, alpha=ALPHA, rmax=RMAX, ads_iterations=30, p_inj=pp[:, 0],
                        p_cont=pp[:, 1], p_abnd=pp[:, 2], epoch_rounds=args.serve_epoch_rounds,
                        preempt_rounds=args.serve_preempt_rounds) as srv:
            # warm-up: one request of each kind (workspaces, graph capture)
            for k in (c2g.REQ_SSSP, c2g.REQ_PPR, c2g.REQ_ADSORPTION):
                t = srv.submit(k, source=int(cand[0]), seeds=rng.choice(V, 16, replace=False) if k == 2 else None)
                srv.wait(t)
            base = srv.stats().completed
            tickets = []
            t_start = time.time()
            t_next = t_start
            for k, gap in zip(kinds, gaps):
                t_next += gap
                while time.time() < t_next:
                    pass
                if k == c2g.REQ_ADSORPTION:
                    tickets.append(srv.submit(k, seeds=rng.choice(V, 16, replace=False)))
                else:
                    tickets.append(srv.submit(k, source=int(rng.choice(cand))))
            lat = []
            for t in tickets:
                st, ms = srv.wait(t)
                assert st == 0, st
                lat.append(ms)
            wall = time.time() - t_start
            stats = srv.stats()
        g.close()
    lat = np.array(lat)
    line = {"mode": "serve", "metric": "serving: queries/s and p50/p99 latency, Poisson arrivals, mix 50/35/15",
            "value": n / wall, "unit": "queries/s", "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic R-MAT (seeded); no public dataset",
            "config": {"workload": "rmat-s%d-ef%d unpruned, %d requests (%d SSSP / %d PPR / %d adsorption)" % (
                args.serve_scale, args.edge_factor, n, kinds.count(0), kinds.count(1), kinds.count(2)),
                "offered_rate_qps": args.serve_rate, "alpha": ALPHA, "rmax": RMAX, "ads_iterations": 30,
                "ads_labels": 16, "epoch_rounds": args.serve_epoch_rounds,
                "preempt_rounds": args.serve_preempt_rounds,
                "admission": "SSSP / PPR requests take free slots of the running batch at every epoch boundary"},
            "detail": {"epochs_or_batches": list(stats.batches), "max_running": stats.max_batch,
                       "admit_cap": list(stats.admit_cap), "evictions": stats.evictions,
                       "completed_after_warmup": stats.completed - base, "gen_s": gen_s, "wall_s": wall}}
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """PPR adjoint throughput (config 4): gradient of the summed PPR score of 64 random
    targets w.r.t. every edge weight, alpha 0.15, eps 1e-8 forward and backward."""
    import c2g

    rng = np.random.default_rng(9)
    with tempfile.TemporaryDirectory(dir=args.workdir) as d:
        c2g.rmat_write(d, args.adjoint_scale, args.edge_factor, 4, 1, 1000)
        vl = c2g.read_array(os.path.join(d, "origin", "vlist.bin"))
        V = len(vl) - 1
        cand = np.flatnonzero(np.diff(vl) > 0)
        with c2g.Graph.load(d, "origin") as g:
            prm = g.ppr_params(alpha=ALPHA, rmax=1e-8, seeded=0, pr0=ALPHA, r0=1.0, max_iter=10000)
            srcs = rng.choice(cand, args.warmup + args.steps, replace=False)
            ms = byt = 0.0
            for i, s in enumerate(srcs):
                targets = rng.choice(V, 64, replace=False).astype(np.int32)
                _, _, _, _, st = g.ppr_adjoint(int(s), targets, prm, rmax_backward=1e-8)
                if i >= args.warmup:
                    ms += st.device_ms
                    byt += st.alg_bytes
            E = g.E
    peak, peak_kind = measured_peak()
    line = {"mode": "adjoint", "metric": "PPR adjoint gradients/s (dL/dw for every edge, 64 targets)",
            "value": args.steps / (ms / 1000.0), "unit": "gradients/s", "ms_per_gradient": ms / args.steps,
            "higher_is_better": True, "n_gpus": 1, "data": "synthetic R-MAT (seeded); no public dataset",
            "config": {"workload": "rmat-s%d-ef%d, %d vertices, %d edges" % (args.adjoint_scale, args.edge_factor, V, E),
                       "alpha": ALPHA, "eps_forward": 1e-8, "eps_backward": 1e-8, "targets": 64},
            "roofline": {"bound": "hbm", "achieved": byt / (ms / 1000.0) / 1e9, "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": byt / (ms / 1000.0) / 1e9 / peak}}
    print(json.dumps(line), flush=True)


def run_adsorption(args):
    """Adsorption label propagation throughput: 16 seed labels, per-vertex p_inj / p_cont /
    p_abnd ~ Dirichlet(1,1,1), 30 iterations, on an unpruned R-MAT graph in HBM."""
    import torch

    import c2g

    rng = np.random.default_rng(11)
    with tempfile.TemporaryDirectory(dir=args.workdir) as d:
        c2g.rmat_write(d, args.scale, args.edge_factor, args.seed, 1, 1000)
        vl = c2g.read_array(os.path.join(d, "origin", "vlist.bin"))
        V = len(vl) - 1
        pp = torch.from_numpy(rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32).T.copy()).cuda()
        Y = torch.empty((V, 16), dtype=torch.float32, device="cuda")
        ms = byt = 0.0
        with c2g.Graph.load(d, "origin") as g:
            for i in range(args.warmup + args.steps):
                seeds = rng.choice(V, 16, replace=False).astype(np.int32)
                st = g.adsorption_device(seeds, pp[0].data_ptr(), pp[1].data_ptr(), pp[2].data_ptr(), Y.data_ptr(),
                                         iterations=30)
                if i >= args.warmup:
                    ms += st.device_ms
                    byt += st.alg_bytes
            E = g.E
    peak, peak_kind = measured_peak()
    gbs = byt / (ms / 1000.0) / 1e9
    line = {"mode": "adsorption", "metric": "adsorption label propagation queries/s (16 labels, 30 iterations)",
            "value": args.steps / (ms / 1000.0), "unit": "queries/s", "ms_per_query": ms / args.steps,
            "higher_is_better": True, "n_gpus": 1, "data": "synthetic R-MAT (seeded); no public dataset",
            "config": {"workload": "rmat-s%d-ef%d unpruned, %d vertices, %d edges" % (args.scale, args.edge_factor, V, E),
                       "labels": 16, "iterations": 30, "p": "Dirichlet(1,1,1) per vertex"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": gbs / peak}}
    print(json.dumps(line), flush=True)


def run_prune(args):
    """purn-ppr on the GPU (c2g_prune_ppr_device) against the sequential pass: one step is
    one pruning of the whole R-MAT graph (origin/ files in, ppr/ files out).  `value` is
    input edges per second of kernel time; `e2e` the same through the C ABI call with the
    files read and written; the CPU baseline is the oracle's sequential pass (oracle/ingest.c
    orc_prune_ppr, one core); the library's own host pass (prune.cpp) is timed beside it,
    and every step's files are compared with it byte for byte.  purn-sssp on the GPU
    (c2g_prune_sssp_device) is timed the same way into `detail.sssp`."""
    import filecmp
    import shutil

    import c2g
    import oracle

    files = ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist")
    with tempfile.TemporaryDirectory(dir=args.workdir) as base:
        host, dev, orc = (os.path.join(base, x) for x in ("host", "dev", "orc"))
        c2g.rmat_write(host, args.scale, args.edge_factor, args.seed, 1, 1000, gpu=True)
        shutil.copytree(host, dev)
        shutil.copytree(host, orc)
        E = len(c2g.read_array(os.path.join(host, "origin", "elist.bin")))
        t0 = time.time()
        c2g.prune_ppr(host, ALPHA)
        host_s = time.time() - t0
        t0 = time.time()
        oracle.prune_ppr(orc, ALPHA)
        orc_s = time.time() - t0
        kern, call, same = [], [], True
        for i in range(args.warmup + args.steps):
            t0 = time.time()
            ms, rounds, ph = c2g.prune_ppr_device(dev, ALPHA, phases=True)
            dt = time.time() - t0
            same = same and all(filecmp.cmp(os.path.join(host, "ppr", f + ".bin"), os.path.join(dev, "ppr", f + ".bin"),
                                            shallow=False) for f in files)
            if i >= args.warmup:
                kern.append(ms / 1000.0)
                call.append(dt)
        same = same and all(filecmp.cmp(os.path.join(host, "ppr", f + ".bin"), os.path.join(orc, "ppr", f + ".bin"),
                                        shallow=False) for f in files)
        # purn-sssp the same way (seven files: the record->vertex sidecar too)
        sfiles = files + ("hvmap",)
        t0 = time.time()
        c2g.prune_sssp(host)
        s_host = time.time() - t0
        t0 = time.time()
        oracle.prune_sssp(orc)
        s_orc = time.time() - t0
        s_kern, s_call, s_same = [], [], True
        for i in range(args.warmup + args.steps):
            t0 = time.time()
            s_ms, s_rounds, s_ph = c2g.prune_sssp_device(dev, phases=True)
            dt = time.time() - t0
            s_same = s_same and all(filecmp.cmp(os.path.join(host, "sssp", f + ".bin"),
                                                os.path.join(dev, "sssp", f + ".bin"), shallow=False) for f in sfiles)
            if i >= args.warmup:
                s_kern.append(s_ms / 1000.0)
                s_call.append(dt)
        s_same = s_same and all(filecmp.cmp(os.path.join(host, "sssp", f + ".bin"), os.path.join(orc, "sssp", f + ".bin"),
                                            shallow=False) for f in sfiles)
        V = len(c2g.read_array(os.path.join(host, "origin", "vlist.bin"))) - 1
    ks, cs = float(np.mean(kern)), float(np.mean(call))
    line = {"mode": "prune", "metric": "purn-ppr input edges pruned per second", "value": E / ks, "unit": "edges/s",
            "ms_per_step": ks * 1000.0, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "n_gpus": 1, "dtype": "int32 / f32 rows, f64 folds", "data": "synthetic R-MAT (seeded); no public dataset",
            "config": {"workload": "rmat-s%d-ef%d, %d vertices, %d edges, alpha %g" % (args.scale, args.edge_factor, V, E,
                                                                                      ALPHA)},
            "e2e": {"value": E / cs, "unit": "edges/s", "s_per_step": cs,
                    "includes": "reading origin/, building the rows, the kernel, writing ppr/"},
            "cpu_baseline": {"value": E / orc_s, "unit": "edges/s", "cores": 1, "kind": "port",
                             "sample": "the whole graph, oracle/ingest.c orc_prune_ppr"},
            "detail": {"host_pass_s": host_s, "oracle_s": orc_s, "device_call_s": cs, "kernel_s": ks, "rounds": rounds,
                       "phase_ms": dict(zip(("plan", "check", "commit", "copy"), ph)),
                       "identical_to_host_pass_and_oracle": bool(same),
                       "sssp": {"kernel_s": float(np.mean(s_kern)), "device_call_s": float(np.mean(s_call)),
                                "host_pass_s": s_host, "oracle_s": s_orc, "rounds": s_rounds,
                                "phase_ms": dict(zip(("plan", "check", "commit", "copy"), s_ph)),
                                "identical_to_host_pass_and_oracle": bool(s_same)}}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--sssp-per-step", type=int, default=256)
    ap.add_argument("--ppr-per-step", type=int, default=256)
    ap.add_argument("--per-query-sample", type=int, default=8)
    ap.add_argument("--delta", type=int, default=0)
    ap.add_argument("--tile", type=int, default=256)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="queries per kind in the CPU-baseline leg (0: one per host thread)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workdir", default=None)
    ap.add_argument("--mode", default="step", choices=["step", "serve", "adjoint", "adsorption", "prune"],
                    help="step: the batched multi-tenant step (headline); serve: the serving loop; "
                         "adjoint: PPR adjoint throughput; adsorption: label propagation throughput; "
                         "prune: purn-ppr on the GPU against the sequential pass")
    ap.add_argument("--serve-scale", type=int, default=24)
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-rate", type=float, default=5000.0)
    ap.add_argument("--serve-epoch-rounds", type=int, default=4)
    ap.add_argument("--serve-preempt-rounds", type=int, default=0)
    ap.add_argument("--adjoint-scale", type=int, default=20)
    args = ap.parse_args()
    rank, world, local_rank = env_rank()
    import __graft_entry__

    if rank == 0:
        __graft_entry__.build()
    if args.mode != "step":
        if rank == 0:
            {"serve": run_serve, "adjoint": run_adjoint, "adsorption": run_adsorption,
             "prune": run_prune}[args.mode](args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        if world > 1 and rank != 0:
            # wait for rank 0's build
            for _ in range(600):
                if os.path.exists(os.path.join(PKG, "lib", "libc2graph.so")):
                    break
                time.sleep(1)
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
