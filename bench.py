#!/usr/bin/env python3
"""Benchmark: exact k-NN queries/s on one GB300 (N=1,000,000 points, d=3, k=16,
L2, leafsize 16, 1,000,000 queries per step; uniform [0,1)^3, data seed 2,
queries seed 3).

A step is one pass of the query hot path over one batch of 1,000,000 queries.

  value   queries/s with queries, tree and outputs resident in HBM: the C-ABI
          kd_query_device call timed with CUDA events on the stream it runs on,
          L2 flushed (a 256 MiB write) before every timed step.
  e2e     the same metric through the C-ABI kd_query with HOST buffers (pinned):
          the 24 MB query upload and the 256 MB (distances + indices) download
          are inside the timed region.
  roofline  algorithmic bytes per launch of the query kernel (per-query node,
          leaf-row and box counts from the oracle's instrumented descent on the
          identical inputs) / its event-timed duration, against the measured
          HBM copy bandwidth.
  cpu_baseline  the oracle (a C restatement of the reference's build + query,
          OpenMP over all host cores) on the same workload.

`--impl reference` times the reference's CPU algorithm (the oracle port: the
Rust crate cannot be built without a Rust toolchain) on the same config.

Under torchrun (N > 1) every rank holds a replica of the tree and queries its
own 1,000,000-query batch (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "kdtree-rs_gb300"))

N_POINTS = 1_000_000
N_QUERIES = 1_000_000
DIM = 3
K = 16
P = 2.0
LEAFSIZE = 16
METRIC = "exact kNN queries/s (N=1M, d=3, k=16, L2)"
WORKLOAD = "plain-scale uniform N=1,000,000 d=3 leafsize=16, 1,000,000 queries/step, k=16, p=2"


def workload(rank: int = 0):
    data = np.random.default_rng(2).uniform(size=(N_POINTS, DIM))
    q = np.random.default_rng(3 + 1000 * rank).uniform(size=(N_QUERIES, DIM))
    return data, q


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def whole_job_rate(local_s, steps, ws, device):
    """Queries/s of the whole job: every rank ran N_QUERIES x steps queries;
    the job took as long as its slowest rank (max over ranks).  Returns
    (rate, slowest seconds)."""
    if ws > 1:
        import torch
        import torch.distributed as dist

        tt = torch.tensor([local_s], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        local_s = float(tt.item())
    return ws * N_QUERIES * steps / local_s, local_s


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(data, q, threads, reps=3):
    """The oracle on the same workload, all host threads (query) -> q/s."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import kdtree_oracle

    t0 = time.perf_counter()
    t = kdtree_oracle.OracleKDTree(data, leafsize=LEAFSIZE, parallel=True)
    build_s = time.perf_counter() - t0
    best = None
    counts = None
    for _ in range(reps):
        t0 = time.perf_counter()
        t.query(q, k=K, p=P, threads=threads)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
        counts = t.last_counts
    return {"qps": len(q) / best, "build_s": build_s, "counts": counts, "tree": t}


def scipy_baseline(data, q, k=None, leafsize=None):
    """SciPy's cKDTree (the reference's own test oracle) on all host cores
    (workers=-1): a sanity number beside the oracle, not the baseline.  None
    when SciPy is not installed."""
    try:
        from scipy.spatial import cKDTree
    except ImportError:
        return None
    k = K if k is None else k
    leafsize = LEAFSIZE if leafsize is None else leafsize
    try:
        t0 = time.perf_counter()
        t = cKDTree(data, leafsize=leafsize)
        build_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        t.query(q, k=k, p=P, workers=-1)
        query_s = time.perf_counter() - t0
    except Exception as e:  # a sanity number only: never fail the bench line over it
        return {"error": f"{type(e).__name__}: {e}"}
    return {"qps": len(q) / query_s, "build_s": build_s, "workers": os.cpu_count()}


def algorithmic_bytes(counts, n_queries):
    """Per-query B_q = 8d + 16k + 8d*S_q + 24*V_q + 16d*X_q summed over the batch
    (V = nodes visited, S = leaf rows scanned, X = boxes evaluated)."""
    visits, scanned, boxes = counts
    return 8 * DIM * n_queries + 16 * K * n_queries + 8 * DIM * scanned + 24 * visits + 16 * DIM * boxes


def count_nodes(n, leafsize=LEAFSIZE):
    """Nodes of the median-split tree over n points (split at n // 2 while
    n > leafsize), as the reference's count_nodes."""
    memo = {}

    def c(m):
        if m <= leafsize:
            return 1
        if m not in memo:
            memo[m] = 1 + c(m // 2) + c(m - m // 2)
        return memo[m]

    return c(n)


def compulsory_bytes(n_queries=N_QUERIES):
    """Bytes one query launch cannot avoid: the queries in, the results out,
    and every tree array the kernel reads once (FP64 rows for the exact
    values, FP32 rows, original indices, 16-byte nodes, FP32 boxes) plus the
    sort's order and landing leaf per query."""
    nodes = count_nodes(N_POINTS)
    tree = N_POINTS * DIM * 8 + N_POINTS * DIM * 4 + N_POINTS * 4 + nodes * 16 + nodes * 2 * DIM * 4
    return n_queries * DIM * 8 + n_queries * K * 16 + tree + n_queries * 8


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        j = json.loads(p.read_text())
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_inputs():
    """The roofline's ncu-measured inputs (profiles/roofline_inputs.json: DRAM
    traffic per launch of the query kernel on this workload, L2 hit rates of it
    and of the build), each with the commit it was measured at and whether the
    kernel's sources have changed since (then the figure is stale)."""
    import hashlib

    p = ROOT / "profiles" / "roofline_inputs.json"
    if not p.exists():
        return None
    j = json.loads(p.read_text())
    for key in ("k_query_packet", "build"):
        e = j.get(key)
        if not e:
            continue
        h = hashlib.sha256()
        for f in e.get("source_files", []):
            h.update((ROOT / f).read_bytes())
        e["stale"] = h.hexdigest()[:16] != e.get("source_sha16")
    return j


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import kdtree_oracle

    threads = kdtree_oracle.max_threads()
    data, q = workload(0)
    t = kdtree_oracle.OracleKDTree(data, leafsize=LEAFSIZE, parallel=True)
    for _ in range(args.warmup):
        t.query(q, k=K, p=P, threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        t.query(q, k=K, p=P, threads=threads)
        times.append(time.perf_counter() - t0)
    qps = len(q) * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (numpy default_rng seeds 2 / 3)",
        "config": {"workload": WORKLOAD, "n_points": N_POINTS, "queries_per_step": N_QUERIES, "d": DIM, "k": K,
                   "p": P, "leafsize": LEAFSIZE, "parallelism": "rank 0 only, all host threads"},
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": "every step is the full 1,000,000-query batch; oracle restatement of the "
                                   "reference (the Rust crate cannot be built here)"},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


PATH_AUTO, PATH_REFERENCE_ORDER, PATH_PACKET, PATH_TENSOR_CORE, PATH_WARP = 0, 1, 2, 3, 4
# kernels one kd_query_device call launches for d=3, k=16 (queries sorted by
# landing leaf: k_landing_leaf, 3 scan kernels, k_scatter_order; k_query_packet)
LAUNCHES_PER_STEP = 6


def gmm_points(rng, centres, n, sigma=0.01):
    return centres[rng.integers(0, len(centres), n)] + sigma * rng.standard_normal((n, centres.shape[1]))


def build_line(build_s, cpu_s, hbm_peak):
    """The build's report: host wall time of kd_build (incl. the upload) and its
    algorithmic bytes -- per split level, every row's box pass (8d B read) and
    the partition's row and index read + write (2 (8d + 4) B) -- over that time."""
    levels, n = 0, N_POINTS
    while n > LEAFSIZE:  # the largest segment at each depth is ceil(n / 2^depth)
        n = (n + 1) // 2
        levels += 1
    b = levels * N_POINTS * (3 * 8 * DIM + 8)
    gbs = b / build_s / 1e9
    pb = (profiled_inputs() or {}).get("build", {})
    return {"gpu_s": build_s, "cpu_oracle_s": cpu_s, "levels": levels, "algorithmic_bytes": b,
            "achieved_gbs": gbs, "frac_of_hbm": gbs / hbm_peak if hbm_peak else None,
            "l2_hit_rate_pct": pb.get("l2_hit_rate_pct_time_weighted"), "l2_stale": pb.get("stale"),
            "note": "host wall time of kd_build incl. the 24 MB upload; oracle build on all host cores; "
                    "the top levels run a chain of dependent launches and the rest one kernel over "
                    "L2-resident data (L2 hit rate: time-weighted over the build's ncu-captured launches), "
                    "so it is launch- and latency-bound, not HBM-bound"}


def path_lib():
    """The library with kd_query_device_path's signature declared."""
    from kdtree import _core

    lib = _core._lib
    P_, u64_, d_ = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    lib.kd_query_device_path.argtypes = [P_, P_, u64_, u64_, d_, ctypes.c_int, d_, d_, P_, P_, P_, ctypes.c_int, P_]
    lib.kd_query_device_path.restype = ctypes.c_int
    return lib


def time_path(lib, tree, dq, k, p, path, reps, torch, stream, survivors=None, warm=True):
    """Mean ms of kd_query_device_path over `reps` calls (events on `stream`),
    after one untimed call unless `warm` is False."""
    n = dq.shape[0]
    od = torch.empty((n, k), dtype=torch.float64, device=dq.device)
    oi = torch.empty((n, k), dtype=torch.int64, device=dq.device)
    P = ctypes.c_void_p

    def call():
        st = lib.kd_query_device_path(tree._h, P(dq.data_ptr()), dq.numel(), k, p, 0, 0.0, 0.0, P(od.data_ptr()),
                                      P(oi.data_ptr()), P(stream.cuda_stream), path,
                                      P(survivors.data_ptr()) if survivors is not None else None)
        if st:
            raise RuntimeError(f"kd_query_device_path failed: {st}")

    if warm:
        call()  # warm-up (and, for the tensor-core path, the one-time BF16 copy of the tree)
    if survivors is not None:
        survivors.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        call()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps, (od, oi)


def plain_scale_cases(lib, torch, stream, dev):
    """Plain scale: N=1M, d=3, leafsize 16, 1M queries; k in {1, 16}, p in {1, 2, inf},
    uniform and a 64-component Gaussian mixture (sigma 0.01)."""
    from kdtree import KDTree

    out = {}
    rd, rq = np.random.default_rng(2), np.random.default_rng(3)
    centres = np.random.default_rng(4).uniform(size=(64, DIM))
    sets = {"uniform": (rd.uniform(size=(N_POINTS, DIM)), rq.uniform(size=(N_QUERIES, DIM))),
            "gmm": (gmm_points(rd, centres, N_POINTS), gmm_points(rq, centres, N_QUERIES))}
    for name, (data, q) in sets.items():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tree = KDTree(data, leafsize=LEAFSIZE)
        build_s = time.perf_counter() - t0
        dq = torch.from_numpy(q).to(dev)
        for k in (1, 16):
            for p in (1.0, 2.0, float("inf")):
                ms, _ = time_path(lib, tree, dq, k, p, PATH_AUTO, 3, torch, stream)
                out[f"{name}-k{k}-p{'inf' if p == float('inf') else int(p)}"] = {"qps": N_QUERIES / ms * 1e3,
                                                                               "ms": ms}
        out[f"{name}-build_s"] = build_s
        del tree
    return out


def precision_cases(lib, torch, stream, dev, cpu_threads):
    """Precision: N=1M, d in {16, 64}, standard normal x per-dimension scale
    log-uniform in [0.1, 10], 100k queries, k=32, L2.  The tensor-core filter
    path against the plain CUDA-core path (the best-first warp traversal: FP32
    filters, exact FP64 values in the reference's summation order), both on all
    100k queries and compared bit for bit; the reference-order warp kernel (the
    reference's own visiting order and FP64 gates) on a sample; the filter's
    survivors per pair and the BF16 score's error against FP64; a sample
    checked against the oracle."""
    from kdtree import KDTree

    out = {}
    for d in (16, 64):
        rng = np.random.default_rng(300 + d)
        scale = np.exp(rng.uniform(np.log(0.1), np.log(10), d))
        data = rng.standard_normal((1_000_000, d)) * scale
        q = rng.standard_normal((100_000, d)) * scale
        t0 = time.perf_counter()
        tree = KDTree(data, leafsize=16)
        build_s = time.perf_counter() - t0
        dq = torch.from_numpy(q).to(dev)
        surv = torch.zeros(3, dtype=torch.int64, device=dev)  # TC survivors, near ties, full reruns
        ms_tc, (od, oi) = time_path(lib, tree, dq, 32, 2.0, PATH_TENSOR_CORE, 3, torch, stream, surv)
        pairs = 3 * q.shape[0] * data.shape[0]
        rerank = int(surv[0].item()) / pairs
        tc_ties = [int(surv[1].item()) / (3 * q.shape[0]), int(surv[2].item()) / (3 * q.shape[0])]
        cnt = torch.zeros(3, dtype=torch.int64, device=dev)
        ms_pl, (pd_, pi_) = time_path(lib, tree, dq, 32, 2.0, PATH_WARP, 1, torch, stream, cnt)
        warp_ties = [int(cnt[1].item()) / q.shape[0], int(cnt[2].item()) / q.shape[0]]
        same = bool(torch.equal(oi, pi_) and torch.equal(od, pd_))
        n_ref = 152 * 4 * 8  # eight warps an SM's worth of queries for the reference-order kernel
        sample = dq[:n_ref].contiguous()
        ms_ref, (rd_, ri_) = time_path(lib, tree, sample, 32, 2.0, PATH_REFERENCE_ORDER, 1, torch, stream)
        same_ref = bool(torch.equal(oi[:n_ref], ri_) and torch.equal(od[:n_ref], rd_))
        # BF16 score error against FP64 on the true neighbours of 200 queries
        c = (data.min(0) + data.max(0)) / 2
        qi = np.repeat(np.arange(200), 32)
        pi = oi[:200].cpu().numpy().reshape(-1)
        qb = torch.from_numpy(q[:200] - c).float().bfloat16().double().numpy()
        pb = torch.from_numpy(data[pi] - c).float().bfloat16().double().numpy()
        approx = (qb[qi] ** 2).sum(1) + (pb ** 2).sum(1) - 2 * (qb[qi] * pb).sum(1)
        exact = ((q[qi] - data[pi]) ** 2).sum(1)
        rel = np.abs(approx - exact) / exact
        tc_qps, plain_qps = q.shape[0] / ms_tc * 1e3, q.shape[0] / ms_pl * 1e3
        case = {"build_s": build_s, "tc_qps": tc_qps, "tc_ms_100k": ms_tc, "plain_qps": plain_qps,
                "plain_path": "warp best-first (CUDA cores, FP64-exact)", "plain_ms_100k": ms_pl,
                "tc_over_plain": tc_qps / plain_qps, "identical": same and same_ref,
                "reference_order_qps": n_ref / ms_ref * 1e3, "reference_order_sample": n_ref,
                "rerank_fraction": rerank, "near_tie_fraction": {"tc": tc_ties, "warp": warp_ties,
                                                            "note": "[flagged, run again in the reference's order]"},
                "filter_rel_err_max": float(rel.max()),
                "filter_rel_err_median": float(np.median(rel))}
        if cpu_threads:
            sys.path.insert(0, str(ROOT / "oracle"))
            import kdtree_oracle

            ot = kdtree_oracle.OracleKDTree(data, leafsize=16, parallel=True)
            ns = 2000 if d == 16 else 300
            t0 = time.perf_counter()
            o_d, o_i = ot.query(q[:ns], k=32, threads=cpu_threads)
            case["cpu_oracle_qps"] = ns / (time.perf_counter() - t0)
            case["cpu_sample"] = ns
            case["identical"] = case["identical"] and bool(
                np.array_equal(o_i, oi[:ns].cpu().numpy()) and np.array_equal(o_d, od[:ns].cpu().numpy()))
        out[f"d{d}"] = case
        del tree
    return out


def batched_jobs(torch, dev):
    """The batched case's draw (256 trees, batched_case): [(d, k, (tree, device queries, k, out_d, out_i))]."""
    from kdtree import KDTree

    rng = np.random.default_rng(400)
    n_trees = 256
    ns = np.exp(rng.uniform(np.log(1e3), np.log(5e5), n_trees)).astype(np.int64)
    ds = rng.choice([2, 3, 8], n_trees)
    qs = np.exp(rng.uniform(np.log(1.0), np.log(5e4), n_trees)).astype(np.int64)
    ks = rng.choice([1, 4, 32], n_trees)
    jobs = []
    for n, d, nq, k in zip(ns, ds, qs, ks):
        tree = KDTree(rng.uniform(size=(int(n), int(d))))
        dq = torch.from_numpy(rng.uniform(size=(int(nq), int(d)))).to(dev)
        jobs.append((int(d), int(k), (tree, dq, int(k), torch.empty((int(nq), int(k)), dtype=torch.float64,
                                                                  device=dev),
                                      torch.empty((int(nq), int(k)), dtype=torch.int64, device=dev))))
    return jobs


def batched_classes(torch, dev, stream, reps=5):
    """The batched case split by (d, k) class: each class's jobs as a plan of their own
    (graph mode, after the tuning run), ms per run and the tuner's choice; the
    whole batch for comparison.  Classes overlap one another in the whole
    batch, so their times add up to more than its time."""
    from kdtree import BatchQuery, _core

    jobs = batched_jobs(torch, dev)

    def timed(js):
        plan = BatchQuery(js)
        for _ in range(2):
            plan.run(stream, _core.BATCH_GRAPH)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            plan.run(stream, _core.BATCH_GRAPH)
        torch.cuda.synchronize()
        s = (time.perf_counter() - t0) / reps
        choice = plan.choice()
        del plan
        return s, choice

    out = {}
    s, choice = timed([j for _, _, j in jobs])
    nq = sum(j[1].shape[0] for _, _, j in jobs)
    out["all"] = {"queries": nq, "ms": s * 1e3, "qps": nq / s, "choice": choice}
    for d in (2, 3, 8):
        for k in (1, 4, 32):
            js = [j for dj, kj, j in jobs if dj == d and kj == k]
            if not js:
                continue
            nq = sum(j[1].shape[0] for j in js)
            s, choice = timed(js)
            out[f"d{d}_k{k}"] = {"jobs": len(js), "queries": nq, "ms": s * 1e3, "qps": nq / s, "choice": choice}
    return out


def batched_case(torch, dev, stream, reps=5):
    """Batched: 256 trees, N log-uniform in [1e3, 5e5], d in {2, 3, 8}, uniform
    [0,1)^d points, leafsize 32 (the reference's default); per tree Q queries,
    Q log-uniform in [1, 5e4], k in {1, 4, 32}, L2; one seed (400) for the whole
    draw.  Total queries/s of the batch plan: one CUDA graph holding the sort
    and ONE persistent query launch, the same launches without the graph, and
    per-tree launches (one kd_query_device launch sequence per tree)."""
    from kdtree import BatchQuery, _core

    t0 = time.perf_counter()
    jobs = [j for _, _, j in batched_jobs(torch, dev)]
    build_s = time.perf_counter() - t0
    plan = BatchQuery(jobs)
    total_q = sum(j[1].shape[0] for j in jobs)
    out = {"trees": len(jobs), "points": sum(j[0].n_points for j in jobs), "queries": total_q, "build_all_s": build_s}
    results = {}
    for name, mode in (("graph", _core.BATCH_GRAPH), ("fused_no_graph", _core.BATCH_FUSED),
                       ("per_tree_launches", _core.BATCH_PER_JOB)):
        for _ in range(2):
            plan.run(stream, mode)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            plan.run(stream, mode)
        s = (time.perf_counter() - t0) / reps
        out[name] = {"qps": total_q / s, "ms": s * 1e3}
        results[name] = [(j[3].clone(), j[4].clone()) for j in jobs[:16]]
        if name == "graph":  # the first graph run tuned the plan
            out["autotuner"] = plan.choice()
    out["identical_across_modes"] = all(
        torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
        for other in ("fused_no_graph", "per_tree_launches") for a, b in zip(results["graph"], results[other]))
    out["speedup_graph_vs_per_tree"] = out["graph"]["qps"] / out["per_tree_launches"]["qps"]
    del plan, jobs
    return out


def serving_case(torch, duration_s=2.0, n_templates=256):
    """Serving: 32 trees, N log-uniform in [1e5, 4e6], d in {3, 8, 16}, each a
    64-component Gaussian mixture (centres uniform in [0,1)^d, sigma 0.01),
    leafsize 32; requests: tree uniform, Q log-uniform in [1, 1e5] queries from
    the tree's mixture, k log-uniform in [1, 64] rounded, L2; seed 500.  Served
    by kdtree.Server (continuous batching).  Peak load: a closed loop keeping 64
    requests in flight for duration_s; then Poisson arrivals at 50/70/90% of that
    rate for duration_s each: p50/p99 latency (submission to completion) and
    sustained queries/s."""
    import threading

    from kdtree import KDTree, Server

    rng = np.random.default_rng(500)
    n_trees = 32
    ns = np.exp(rng.uniform(np.log(1e5), np.log(4e6), n_trees)).astype(np.int64)
    ds = rng.choice([3, 8, 16], n_trees)
    trees, centres = [], []
    t0 = time.perf_counter()
    for n, d in zip(ns, ds):
        c = rng.uniform(size=(64, int(d)))
        data = c[rng.integers(0, 64, int(n))] + 0.01 * rng.standard_normal((int(n), int(d)))
        trees.append(KDTree(data))
        centres.append(c)
        del data
    build_s = time.perf_counter() - t0
    templates = []
    for _ in range(n_templates):
        ti = int(rng.integers(n_trees))
        nq = max(1, int(np.exp(rng.uniform(0.0, np.log(1e5)))))
        k = max(1, int(round(np.exp(rng.uniform(0.0, np.log(64))))))
        d = int(ds[ti])
        q = centres[ti][rng.integers(0, 64, nq)] + 0.01 * rng.standard_normal((nq, d))
        qp = torch.from_numpy(q).pin_memory().numpy()
        od = torch.empty((nq, k), dtype=torch.float64).pin_memory().numpy()
        oi = torch.empty((nq, k), dtype=torch.int64).pin_memory().numpy()
        templates.append((ti, qp, k, od, oi))
    srv = Server(trees)
    # warm-up, and three requests checked against lone KDTree.query calls
    tickets = [srv.submit(ti, q, k, out=(od, oi)) for ti, q, k, od, oi in templates]
    for tk in tickets:
        srv.wait(tk)
    identical = True
    for ti, q, k, od, oi in templates[:3]:
        d_, i_ = trees[ti].query(q, k=k)
        identical &= bool(np.array_equal(d_.view(np.int64), od.view(np.int64)) and np.array_equal(i_, oi))
    total_q = sum(t[1].shape[0] for t in templates)

    def run_load(rate, duration, window=None):
        """Submit requests at Poisson times (rate/s, for `duration` s), or -- with
        `window` -- keep that many in flight as fast as the server allows, until
        `duration` s have passed; return (latencies, queries done, elapsed)."""
        busy = [False] * n_templates
        cv = threading.Condition()
        pending, lat, lat_nq, done_q, finished = [], [], [], [0], [False]

        def waiter():
            while True:
                with cv:
                    while not pending and not finished[0]:
                        cv.wait()
                    if not pending:
                        return
                    tk, j = pending.pop(0)
                _, _, l = srv.wait(tk)
                with cv:
                    busy[j] = False
                    lat.append(l)
                    lat_nq.append(templates[j][1].shape[0])
                    done_q[0] += templates[j][1].shape[0]
                    cv.notify_all()

        th = threading.Thread(target=waiter)
        th.start()
        t_start = time.perf_counter()
        t_next = t_start
        n_sub = 0
        while True:
            if window is None:
                t_next += rng.exponential(1.0 / rate)
                if t_next - t_start > duration:
                    break
                while time.perf_counter() < t_next:
                    pass
            elif time.perf_counter() - t_start > duration:
                break
            with cv:
                # a template's buffers serve one request at a time; with `window`,
                # at most that many requests are in flight
                while all(busy) or (window is not None and sum(busy) >= window):
                    cv.wait()
                j = int(rng.integers(0, n_templates))
                while busy[j]:
                    j = (j + 1) % n_templates
                busy[j] = True
            ti, q, k, od, oi = templates[j]
            tk = srv.submit(ti, q, k, out=(od, oi))
            n_sub += 1
            with cv:
                pending.append((tk, j))
                cv.notify_all()
        with cv:
            finished[0] = True
            cv.notify_all()
        th.join()
        return np.array(lat) * 1e3, done_q[0], time.perf_counter() - t_start, np.array(lat_nq)

    # peak: a closed loop keeping 64 requests in flight for 2 s
    lat, q_done, el, _ = run_load(None, duration_s, window=64)
    peak_rps = len(lat) / el
    out = {"trees": n_trees, "points": int(ns.sum()), "build_all_s": build_s, "templates": n_templates,
           "mean_queries_per_request": total_q / n_templates, "identical_to_lone_queries": identical,
           "peak": {"requests_per_s": peak_rps, "queries_per_s": q_done / el, "in_flight": 64,
                    "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}}
    for frac in (0.5, 0.7, 0.9):
        rate = frac * peak_rps
        lat, q_done, el, nqs = run_load(rate, duration_s)
        small = lat[nqs <= 10_000]
        out[f"load_{int(frac * 100)}"] = {"offered_requests_per_s": rate, "requests": len(lat),
                                          "p50_ms": float(np.percentile(lat, 50)),
                                          "p99_ms": float(np.percentile(lat, 99)),
                                          "p50_ms_le_10k": float(np.percentile(small, 50)) if len(small) else None,
                                          "p99_ms_le_10k": float(np.percentile(small, 99)) if len(small) else None,
                                          "requests_le_10k": int(len(small)),
                                          "sustained_queries_per_s": q_done / el}
    srv.close()
    del trees
    return out


def grid_case(lib, torch, stream, dev, cpu_threads):
    """The reference's small-size grid (tests/benchmark.py, benches/grid.rs):
    d in {3, 8, 16}, N = 10,000, Q = 1,000, k = 1 -- the GPU build and query
    times (host wall time of the synchronous C-ABI call, inputs in HBM for the
    query) beside the oracle on all host cores."""
    sys.path.insert(0, str(ROOT / "tests"))
    from grid_workloads import build_cases, make_data, make_queries, query_cases

    from kdtree import KDTree

    out = {}
    okd = None
    if cpu_threads:
        sys.path.insert(0, str(ROOT / "oracle"))
        import kdtree_oracle as okd
    for name, d, n, dist in build_cases():
        data = make_data(dist, n, d)
        KDTree(data, leafsize=16)
        t0 = time.perf_counter()
        for _ in range(5):
            KDTree(data, leafsize=16)
        case = {"gpu_ms": (time.perf_counter() - t0) / 5 * 1e3}
        if okd:
            t0 = time.perf_counter()
            okd.OracleKDTree(data, leafsize=16)
            case["cpu_ms"] = (time.perf_counter() - t0) * 1e3
        out[name] = case
    P = ctypes.c_void_p
    for name, d, n, q, dist, leaf, p in query_cases():
        data = make_data(dist, n, d)
        qs = make_queries(q, d)
        tree = KDTree(data, leafsize=leaf)
        dq = torch.from_numpy(qs).to(dev)
        od = torch.empty((q, 1), dtype=torch.float64, device=dev)
        oi = torch.empty((q, 1), dtype=torch.int64, device=dev)

        def call():
            st = lib.kd_query_device(tree._h, P(dq.data_ptr()), dq.numel(), 1, p, 0, 0.0, 0.0, P(od.data_ptr()),
                                     P(oi.data_ptr()), P(stream.cuda_stream))
            if st:
                raise RuntimeError("kd_query_device failed")

        call()
        t0 = time.perf_counter()
        for _ in range(10):
            call()
        case = {"gpu_ms": (time.perf_counter() - t0) / 10 * 1e3}
        if okd:
            ot = okd.OracleKDTree(data, leafsize=leaf)
            t0 = time.perf_counter()
            ot.query(qs, k=1, p=p, threads=cpu_threads)
            case["cpu_ms"] = (time.perf_counter() - t0) * 1e3
        out[name] = case
    return out


def _sig(x, n=4):
    """x rounded to n significant digits (for the compact case summary)."""
    if isinstance(x, bool) or x is None:
        return x
    if isinstance(x, float):
        return float(f"{x:.{n}g}")
    return x


def compact_cases(cases):
    """The secondary workloads' headline numbers, short enough to stay inside
    the last 1,500 characters of the bench output (the full details go to
    stderr as one JSON line)."""
    out = {}
    ps = cases.get("plain_scale")
    if ps:
        k1 = [v["qps"] for key, v in ps.items() if isinstance(v, dict) and "-k1-" in key]
        k16 = [v["qps"] for key, v in ps.items() if isinstance(v, dict) and "-k16-" in key]
        out["plain_scale"] = {"k1_qps_min_max": [_sig(min(k1), 3), _sig(max(k1), 3)],
                              "k16_qps_min_max": [_sig(min(k16), 3), _sig(max(k16), 3)],
                              "build_s": [_sig(ps.get("uniform-build_s"), 3), _sig(ps.get("gmm-build_s"), 3)]}
    pr = cases.get("precision")
    if pr:
        out["precision"] = {d: {k: _sig(v, 3) for k, v in c.items()
                                if k in ("tc_qps", "plain_qps", "tc_over_plain", "reference_order_qps",
                                         "cpu_oracle_qps", "identical", "rerank_fraction")}
                            for d, c in pr.items()}
    ba = cases.get("batched")
    if ba:
        out["batched"] = {"graph_qps": _sig(ba["graph"]["qps"], 3),
                          "per_tree_qps": _sig(ba["per_tree_launches"]["qps"], 3),
                          "identical": ba.get("identical_across_modes"), "autotuner": ba.get("autotuner")}
    sv = cases.get("serving")
    if sv:
        out["serving"] = {"peak_qps": _sig(sv["peak"]["queries_per_s"], 3),
                          "identical": sv.get("identical_to_lone_queries")}
        for key in ("load_50", "load_70", "load_90"):
            if key in sv:
                out["serving"][key] = {k: _sig(sv[key][k], 3) for k in sv[key]
                                       if k in ("p50_ms", "p99_ms", "p99_ms_le_10k")}
    gr = cases.get("grid")
    if gr:
        q = [v for key, v in gr.items() if key.startswith("query-") and "cpu_ms" in v]
        out["grid"] = {"query_cases": len(q), "faster_than_cpu": sum(v["gpu_ms"] < v["cpu_ms"] for v in q)}
    return out


PROFILE_CASES = {
    "build": "kd_build, N=1,000,000 uniform d=3, leafsize 16 (every build kernel)",
    "packet": "packet traversal, N=1M uniform d=3 leafsize 16, 200,000 queries, k=16 (with the landing-leaf sort)",
    "warp16": "best-first warp, 64-component mixture d=16 sigma 0.01, N=1M, 20,000 queries, k=16",
    "warpdyn": "best-first warp at a runtime width, normal d=20, N=200,000, 20,000 queries, k=8",
    "ref": "reference-order warp kernel, eps=0.5, N=1M uniform d=3, 100,000 queries, k=16",
    "onethread": "one-thread reference-order kernel (k > 64), N=1M uniform d=3, 20,000 queries, k=100",
    "tc": "tensor-core filter, scaled normal d=64, N=100,000, 19,456 queries, k=32",
    "batch": "batch plan: 64 trees N log-uniform [1e3, 2e5], d in {2,3,8}, 100k queries in all, k in {1,4,32}",
}


def run_profile_case(name):
    """One small scenario per kernel family, the target of the per-kernel ncu
    captures summarised under profiles/ (one kernel, one launch each)."""
    import torch

    from kdtree import BatchQuery, KDTree

    lib = path_lib()
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(77)
    out = {"case": name}
    cnt = torch.zeros(3, dtype=torch.int64, device="cuda")  # TC survivors, near ties, full reruns (timed call)
    t0 = time.perf_counter()
    if name == "build":
        data = np.random.default_rng(2).uniform(size=(N_POINTS, 3))
        KDTree(data, leafsize=16)
    elif name in ("packet", "ref", "onethread"):
        data = np.random.default_rng(2).uniform(size=(N_POINTS, 3))
        tree = KDTree(data, leafsize=16)
        nq = {"packet": 200_000, "ref": 100_000, "onethread": 20_000}[name]
        dq = torch.from_numpy(np.random.default_rng(3).uniform(size=(nq, 3))).cuda()
        if name == "packet":
            out["ms"] = time_path(lib, tree, dq, 16, 2.0, PATH_PACKET, 1, torch, stream, cnt)[0]
        elif name == "onethread":
            out["ms"] = time_path(lib, tree, dq, 100, 2.0, PATH_AUTO, 1, torch, stream, cnt)[0]
        else:
            od = torch.empty((nq, 16), dtype=torch.float64, device="cuda")
            oi = torch.empty((nq, 16), dtype=torch.int64, device="cuda")
            P = ctypes.c_void_p
            st = lib.kd_query_device(tree._h, P(dq.data_ptr()), dq.numel(), 16, 2.0, 0, 0.0, 0.5, P(od.data_ptr()),
                                     P(oi.data_ptr()), P(stream.cuda_stream))
            torch.cuda.synchronize()
            assert st == 0
    elif name == "warp16":
        c = rng.uniform(size=(64, 16))
        data = c[rng.integers(0, 64, N_POINTS)] + 0.01 * rng.standard_normal((N_POINTS, 16))
        q = c[rng.integers(0, 64, 20_000)] + 0.01 * rng.standard_normal((20_000, 16))
        tree = KDTree(data)
        out["ms"] = time_path(lib, tree, torch.from_numpy(q).cuda(), 16, 2.0, PATH_WARP, 1, torch, stream, cnt)[0]
    elif name == "warpdyn":
        data = rng.standard_normal((200_000, 20))
        q = rng.standard_normal((20_000, 20))
        tree = KDTree(data, leafsize=16)
        out["ms"] = time_path(lib, tree, torch.from_numpy(q).cuda(), 8, 2.0, PATH_WARP, 1, torch, stream, cnt)[0]
    elif name == "tc":
        scale = np.exp(rng.uniform(np.log(0.1), np.log(10), 64))
        data = rng.standard_normal((100_000, 64)) * scale
        q = rng.standard_normal((152 * 128, 64)) * scale
        tree = KDTree(data, leafsize=16)
        out["ms"] = time_path(lib, tree, torch.from_numpy(q).cuda(), 32, 2.0, PATH_TENSOR_CORE, 1, torch, stream, cnt)[0]
    elif name == "batch":
        jobs = []
        for _ in range(64):
            n = int(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))
            d = int(rng.choice([2, 3, 8]))
            nq = int(np.exp(rng.uniform(np.log(100), np.log(5000))))
            k = int(rng.choice([1, 4, 32]))
            jobs.append((KDTree(rng.uniform(size=(n, d))), torch.from_numpy(rng.uniform(size=(nq, d))).cuda(), k,
                         torch.empty((nq, k), dtype=torch.float64, device="cuda"),
                         torch.empty((nq, k), dtype=torch.int64, device="cuda")))
        BatchQuery(jobs).run(stream, 1)  # the fused launches, no graph (the graph's first run tunes)
    else:
        raise SystemExit(f"unknown profile case {name!r}; cases: {', '.join(PROFILE_CASES)}")
    torch.cuda.synchronize()
    out["wall_s"] = time.perf_counter() - t0
    out["near_ties"] = [int(cnt[1].item()), int(cnt[2].item())]
    print(json.dumps(out), flush=True)
    return 0


WORK_NAMES = ["warps", "live_queries", "seed_rows", "node_pops", "nodes_entered", "lane_nodes_needed",
              "leaves_scanned", "rows_scanned", "lane_rows_needed", "rows_past_filter", "offers",
              "cycles_setup_and_seed", "cycles_nodes", "cycles_leaf_filter", "cycles_offers", "cycles_sort_write"]


def run_work_counts():
    """The packet traversal's work on the bench workload (uniform N=1M, d=3,
    k=16, 1M queries), counted by the measurement build of the library
    (KD_WORK_COUNTS), against the oracle's per-query work of the reference's
    own descent (nodes visited V_q, rows scanned S_q)."""
    import torch

    sys.path.insert(0, str(ROOT / "kdtree-rs_gb300"))
    import build_lib

    L = ctypes.CDLL(str(build_lib.build(counting=True)))
    VP, u64, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    L.kd_build.argtypes = [VP, u64, u64, u64, ctypes.c_int, ctypes.POINTER(VP)]
    L.kd_query_device_path.argtypes = [VP, VP, u64, u64, dbl, ctypes.c_int, dbl, dbl, VP, VP, VP, ctypes.c_int, VP]
    L.kd_work_counts.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int, ctypes.c_int]
    L.kd_free.argtypes = [VP]
    data, q = workload(0)
    h = VP()
    assert L.kd_build(VP(data.ctypes.data), data.size, DIM, LEAFSIZE, 0, ctypes.byref(h)) == 0
    dq = torch.from_numpy(q).cuda()
    od = torch.empty((len(q), K), dtype=torch.float64, device="cuda")
    oi = torch.empty((len(q), K), dtype=torch.int64, device="cuda")
    buf = (ctypes.c_ulonglong * 16)()
    assert L.kd_work_counts(buf, 16, 1) == 0  # reset
    assert L.kd_query_device_path(h, VP(dq.data_ptr()), dq.numel(), K, P, 0, 0.0, 0.0, VP(od.data_ptr()),
                                  VP(oi.data_ptr()), None, PATH_PACKET, None) == 0
    assert L.kd_work_counts(buf, 16, 0) == 0
    c = dict(zip(WORK_NAMES, [int(x) for x in buf[:len(WORK_NAMES)]]))
    cyc = {k: v for k, v in c.items() if k.startswith("cycles_")}
    tot = sum(cyc.values()) or 1
    L.kd_free(h)
    sys.path.insert(0, str(ROOT / "oracle"))
    import kdtree_oracle

    ot = kdtree_oracle.OracleKDTree(data, leafsize=LEAFSIZE, parallel=True)
    ot.query(q, k=K, p=P, threads=os.cpu_count())
    v_q, s_q = ot.last_counts[0] / len(q), ot.last_counts[1] / len(q)
    nq, w = c["live_queries"], c["warps"]
    rows_lane = (c["rows_scanned"] + 0.0) / w + c["seed_rows"] / nq  # rows a lane evaluates
    out = {"work_counts": c, "per_query": {
        "reference_nodes_visited": v_q, "reference_rows_scanned": s_q,
        "rows_evaluated_per_lane": rows_lane, "rows_needed_per_query": (c["lane_rows_needed"] + c["seed_rows"]) / nq,
        "nodes_entered_per_warp": c["nodes_entered"] / w, "node_pops_per_warp": c["node_pops"] / w,
        "lane_nodes_needed_per_query": c["lane_nodes_needed"] / nq,
        "leaves_scanned_per_warp": c["leaves_scanned"] / w, "offers_per_query": c["offers"] / nq,
        "rows_past_filter_per_query": c["rows_past_filter"] / nq},
        "phase_share": {k[len("cycles_"):]: v / tot for k, v in cyc.items()},
        "inflation": {"rows_evaluated_over_reference": rows_lane / s_q,
                      "rows_needed_over_reference": (c["lane_rows_needed"] + c["seed_rows"]) / nq / s_q,
                      "lane_utilisation_in_leaves": c["lane_rows_needed"] / max(1, 32 * c["rows_scanned"]),
                      "nodes_entered_per_warp_over_reference": c["nodes_entered"] / w / v_q}}
    print(json.dumps(out), flush=True)
    return 0


def run_profile_tc():
    """A tensor-core-path case small enough for an ncu capture: one CTA-filling
    batch (152 x 128 queries) against 100,000 points, d=64, k=32."""
    import torch

    from kdtree import KDTree

    lib = path_lib()
    rng = np.random.default_rng(364)
    scale = np.exp(rng.uniform(np.log(0.1), np.log(10), 64))
    data = rng.standard_normal((100_000, 64)) * scale
    q = rng.standard_normal((152 * 128, 64)) * scale
    tree = KDTree(data, leafsize=16)
    stream = torch.cuda.Stream()
    dq = torch.from_numpy(q).cuda()
    ms, _ = time_path(lib, tree, dq, 32, 2.0, PATH_TENSOR_CORE, 3, torch, stream)
    print(json.dumps({"profile_tc_ms": ms, "queries": q.shape[0], "points": data.shape[0], "d": 64, "k": 32}))
    return 0


def run_profile_warp():
    """A warp-per-query case small enough for an ncu capture: a 64-component
    Gaussian mixture (sigma 0.01) in d=16, N=1,000,000, leafsize 32, 20,000
    queries from the same mixture, k=16, L2; 3 calls."""
    import torch

    from kdtree import KDTree

    lib = path_lib()
    rng = np.random.default_rng(716)
    c = rng.uniform(size=(64, 16))
    data = c[rng.integers(0, 64, 1_000_000)] + 0.01 * rng.standard_normal((1_000_000, 16))
    q = c[rng.integers(0, 64, 20_000)] + 0.01 * rng.standard_normal((20_000, 16))
    tree = KDTree(data)
    stream = torch.cuda.Stream()
    dq = torch.from_numpy(q).cuda()
    ms, _ = time_path(lib, tree, dq, 16, 2.0, PATH_WARP, 3, torch, stream)
    print(json.dumps({"profile_warp_ms": ms, "queries": q.shape[0], "points": data.shape[0], "d": 16, "k": 16}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-cases", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--batched-only", action="store_true", help="only run the batched multi-tree case")
    ap.add_argument("--batched-classes", action="store_true",
                    help="only run the batched multi-tree case split by (d, k) class, one plan per class")
    ap.add_argument("--serving-only", action="store_true", help="only run the serving case")
    ap.add_argument("--precision-only", action="store_true",
                    help="only run the precision case (d=16 and d=64, tensor-core vs FP64 paths), no CPU leg")
    ap.add_argument("--profile-warp", action="store_true",
                    help="only run the warp-per-query path on a profiling-sized case (d=16 mixture, N=1M, "
                         "20,000 queries, k=16), 3 calls")
    ap.add_argument("--profile-tc", action="store_true",
                    help="only run the tensor-core path on a profiling-sized case (N=100k, d=64, "
                         "19,456 queries, k=32), 3 calls")
    ap.add_argument("--work-counts", action="store_true",
                    help="count the packet traversal's work with the measurement build and print it")
    ap.add_argument("--profile-case", default=None,
                    help="only run one small scenario for a per-kernel ncu capture: " + ", ".join(PROFILE_CASES))
    args = ap.parse_args()
    if args.work_counts:
        return run_work_counts()
    if args.profile_case:
        return run_profile_case(args.profile_case)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_tc:
        return run_profile_tc()
    if args.profile_warp:
        return run_profile_warp()
    if args.serving_only:
        import torch

        print(json.dumps({"serving": serving_case(torch)}), flush=True)
        return 0
    if args.precision_only:
        import torch

        stream = torch.cuda.Stream()
        dev = torch.device("cuda", 0)
        print(json.dumps({"precision": precision_cases(path_lib(), torch, stream, dev, 0)}), flush=True)
        return 0
    if args.batched_classes:
        import torch

        stream = torch.cuda.Stream()
        print(json.dumps({"batched_classes": batched_classes(torch, torch.device("cuda", 0), stream)}), flush=True)
        return 0
    if args.batched_only:
        import torch

        stream = torch.cuda.Stream()
        print(json.dumps({"batched": batched_case(torch, torch.device("cuda", 0), stream)}), flush=True)
        return 0

    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from kdtree import KDTree
    from kdtree import _core

    lib = path_lib()
    data, q = workload(rank)

    # build (GPU), timed on the host around the synchronous call
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tree = KDTree(data, leafsize=LEAFSIZE)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    tree = KDTree(data, leafsize=LEAFSIZE)
    build_s = min(build_s, time.perf_counter() - t0)

    dev = torch.device("cuda", local)
    dq = torch.from_numpy(q).to(dev)
    dd = torch.empty((N_QUERIES, K), dtype=torch.float64, device=dev)
    di = torch.empty((N_QUERIES, K), dtype=torch.int64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    def step():
        st = lib.kd_query_device(tree._h, ctypes.c_void_p(dq.data_ptr()), dq.numel(), K, P, 0, 0.0, 0.0,
                                 ctypes.c_void_p(dd.data_ptr()), ctypes.c_void_p(di.data_ptr()),
                                 ctypes.c_void_p(stream.cuda_stream))
        if st:
            raise RuntimeError(f"kd_query_device failed: {st} {_core._last_error()}")

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            flush.zero_()
            step()
    torch.cuda.synchronize()

    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    lib.kd_last_query_kernel_ms.restype = ctypes.c_double
    kernel_ms = []
    with sampler:
        t_wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for e0, e1 in events:
                flush.zero_()
                e0.record(stream)
                step()
                e1.record(stream)
                kernel_ms.append(lib.kd_last_query_kernel_ms())  # step() returned: its kernel is done
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if ws > 1:
        dist.barrier()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in events]
    value, total_s = whole_job_rate(sum(step_ms) / 1e3, args.steps, ws, dev)
    clocks = sampler.summary()
    # the queries the traversal flagged as near ties and ran again in the
    # reference's order: one more (untimed) call of the same step
    cnt = torch.zeros(3, dtype=torch.int64, device=dev)
    time_path(lib, tree, dq, K, 2.0, PATH_AUTO, 1, torch, stream, cnt, warm=False)
    near_ties = {"flagged": int(cnt[1].item()), "rerun_in_reference_order": int(cnt[2].item())}

    # end to end through the C ABI with pinned host buffers
    hq = torch.from_numpy(q).pin_memory()
    hd = torch.empty((N_QUERIES, K), dtype=torch.float64).pin_memory()
    hi = torch.empty((N_QUERIES, K), dtype=torch.int64).pin_memory()

    def e2e_step():
        st = lib.kd_query(tree._h, ctypes.c_void_p(hq.data_ptr()), hq.numel(), K, P, 0, 0.0, 0.0, 0,
                          ctypes.c_void_p(hd.data_ptr()), ctypes.c_void_p(hi.data_ptr()))
        if st:
            raise RuntimeError(f"kd_query failed: {st} {_core._last_error()}")

    for _ in range(max(args.warmup, 3)):
        e2e_step()
    torch.cuda.synchronize()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    e2e_value, e2e_s = whole_job_rate(sum(e2e_times), args.steps, ws, dev)

    # the drop-in surface: KDTree.query with a pageable numpy array in and
    # fresh numpy arrays out (src/lib.rs:161-182)
    for _ in range(2):
        tree.query(q, k=K)
    np_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = tree.query(q, k=K)
        np_times.append(time.perf_counter() - t0)
        del res
    e2e_numpy_value, _ = whole_job_rate(sum(np_times), args.steps, ws, dev)

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return 0

    # CPU baseline (rank 0, N=1 only) and the per-query work counts
    cpu = None
    counts = None
    if not args.no_cpu and ws == 1:
        sys.path.insert(0, str(ROOT / "oracle"))
        import kdtree_oracle

        threads = kdtree_oracle.max_threads()
        cpu = cpu_baseline(data, q, threads)
        counts = cpu["counts"]
    peak, peak_kind = measured_peak()
    roofline = None
    if counts:
        per_launch = algorithmic_bytes(counts, N_QUERIES)
        # the query kernel's own device time (CUDA events the library records on
        # the launching stream around it), averaged over the timed steps
        mean_s = (sum(kernel_ms) / len(kernel_ms) / 1e3) if min(kernel_ms) > 0 else total_s / args.steps
        achieved = per_launch / mean_s / 1e9
        prof = profiled_inputs() or {}
        pk = prof.get("k_query_packet", {})
        traffic = pk.get("traffic_bytes_per_launch")
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": traffic, "peak_kind": peak_kind,
                    "algorithmic_bytes_per_launch": per_launch,
                    "per_query": {"nodes_visited": counts[0] / N_QUERIES, "rows_scanned": counts[1] / N_QUERIES,
                                  "boxes_evaluated": counts[2] / N_QUERIES},
                    "near_ties": near_ties,
                    "compulsory_bytes_per_launch": compulsory_bytes(),
                    "traffic_over_compulsory": (traffic / compulsory_bytes()) if traffic else None,
                    "kernel": "k_query_packet<L2, d=3, K=16>", "kernel_ms": mean_s * 1e3,
                    "traffic_note": "DRAM read+write bytes per launch from ncu on this workload",
                    "traffic_source": {"file": "profiles/roofline_inputs.json", "commit": pk.get("commit", prof.get("commit")),
                                       "stale": pk.get("stale")},
                    "l2_hit_rate_pct": pk.get("l2_hit_rate_pct")}
    line = {
        "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (numpy default_rng: data seed 2, queries seed 3)",
        "config": {"workload": WORKLOAD, "n_points": N_POINTS, "queries_per_step": N_QUERIES, "d": DIM, "k": K,
                   "p": P, "leafsize": LEAFSIZE, "l2": "flushed (256 MiB write) before every timed step",
                   "parallelism": f"replicas x{ws}"},
        "gpu_launches": LAUNCHES_PER_STEP * args.steps,
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(q.nbytes),
                "d2h_bytes_per_step": int(N_QUERIES * K * 16), "api": "kd_query, page-locked host buffers"},
        "e2e_numpy": {"value": e2e_numpy_value, "unit": "queries/s", "h2d_bytes_per_step": int(q.nbytes),
                      "d2h_bytes_per_step": int(N_QUERIES * K * 16),
                      "api": "KDTree.query, pageable numpy in, fresh numpy arrays out"},
        "roofline": roofline,
        "build": build_line(build_s, cpu["build_s"] if cpu else None, peak),
        "cpu_baseline": None if cpu is None else {
            "value": cpu["qps"], "unit": "queries/s", "cores": kdtree_oracle.max_threads(), "kind": "port",
            "sample": "the full 1,000,000-query step, best of 3 runs (oracle restatement of the reference)",
            "scipy_ckdtree": scipy_baseline(data, q)},
        "wall_s_timed_region": t_wall,
    }
    if not args.no_cases and ws == 1:
        ct = None
        if not args.no_cpu:
            ct = kdtree_oracle.max_threads()
        cases = {}
        for name, fn in (("plain_scale", lambda: plain_scale_cases(lib, torch, stream, dev)),
                         ("precision", lambda: precision_cases(lib, torch, stream, dev, ct)),
                         ("grid", lambda: grid_case(lib, torch, stream, dev, ct)),
                         ("batched", lambda: batched_case(torch, dev, stream)),
                         ("serving", lambda: serving_case(torch))):
            t0 = time.perf_counter()
            cases[name] = fn()
            print(f"[bench] case {name}: {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
        print("[bench] cases " + json.dumps(cases), file=sys.stderr, flush=True)
        line["cases"] = compact_cases(cases)  # last key: it ends the output
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
