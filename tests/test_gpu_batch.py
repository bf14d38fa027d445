"""Batched queries over many trees (kd_batch_*): every job's results equal a
kd_query_device call on the same job, bit for bit, in every run mode (one CUDA
graph with one persistent launch, the same launches without a graph, per-job
launches), on replay with new query contents, and with jobs outside the packet
traversal (other widths, k > 32, general L^p, eps > 0) mixed in."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bit_exact

pytestmark = pytest.mark.gpu


def _jobs(rng, specs, torch):
    from kdtree import KDTree

    jobs, host = [], []
    for n, d, nq, k in specs:
        data = rng.uniform(size=(n, d))
        q = rng.uniform(size=(nq, d)) * 1.1 - 0.05  # a few queries outside the root box
        t = KDTree(data, leafsize=int(rng.choice([8, 16, 32])))
        dq = torch.from_numpy(q).cuda()
        od = torch.full((nq, k), -1.0, dtype=torch.float64, device="cuda")
        oi = torch.full((nq, k), -1, dtype=torch.int64, device="cuda")
        jobs.append((t, dq, k, od, oi))
        host.append((data, q))
    return jobs, host


def _single(job, p=2.0, max_distance=None, eps=0.0):
    import torch

    from kdtree import _core

    t, dq, k, _, _ = job
    L = _core._lib
    od = torch.empty((dq.shape[0], k), dtype=torch.float64, device="cuda")
    oi = torch.empty((dq.shape[0], k), dtype=torch.int64, device="cuda")
    P = ctypes.c_void_p
    st = L.kd_query_device(t._h, P(dq.data_ptr()), dq.numel(), k, p, int(max_distance is not None),
                           float(max_distance or 0.0), eps, P(od.data_ptr()), P(oi.data_ptr()), None)
    assert st == 0, _core._last_error()
    return od.cpu().numpy(), oi.cpu().numpy()


SPECS = [
    (20_000, 3, 5000, 16), (3000, 2, 700, 1), (50_000, 8, 2000, 32), (1000, 3, 1, 4), (8000, 2, 3000, 8),
    (40_000, 3, 33, 5), (6000, 8, 900, 1), (12_000, 5, 400, 6), (9000, 3, 600, 40), (2000, 16, 300, 10),
]


@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
def test_batch_modes_match_single_calls(oracle, p):
    import torch

    from kdtree import BatchQuery, _core

    rng = np.random.default_rng(int(7 + (p if np.isfinite(p) else 9)))
    jobs, host = _jobs(rng, SPECS, torch)
    ref = [_single(j, p=p) for j in jobs]
    plan = BatchQuery(jobs, p=p)
    for mode in (_core.BATCH_GRAPH, _core.BATCH_FUSED, _core.BATCH_PER_JOB, _core.BATCH_GRAPH):
        for _, _, _, od, oi in jobs:
            od.fill_(-1.0)
            oi.fill_(-1)
        plan.run(mode=mode)
        for (t, dq, k, od, oi), r in zip(jobs, ref):
            assert_bit_exact((od.cpu().numpy(), oi.cpu().numpy()), r)
    # spot-check against the oracle
    for (t, dq, k, od, oi), (data, q) in list(zip(jobs, host))[:4]:
        o = oracle.OracleKDTree(data, leafsize=t.leafsize).query(q, k=k, p=p, parallel=True)
        assert_bit_exact((od.cpu().numpy(), oi.cpu().numpy()), o)


def test_batch_replay_follows_new_queries():
    import torch

    from kdtree import BatchQuery

    rng = np.random.default_rng(3)
    jobs, _ = _jobs(rng, SPECS[:5], torch)
    plan = BatchQuery(jobs)
    plan.run()
    for _, dq, _, _, _ in jobs:
        dq.copy_(torch.from_numpy(rng.uniform(size=tuple(dq.shape))))
    plan.run()
    for j in jobs:
        assert_bit_exact((j[3].cpu().numpy(), j[4].cpu().numpy()), _single(j))


def test_batch_eps_and_max_distance():
    import torch

    from kdtree import BatchQuery

    rng = np.random.default_rng(5)
    jobs, _ = _jobs(rng, SPECS[:6], torch)
    for kw in ({"eps": 0.5}, {"max_distance": 0.02}, {"p": 3.0}):
        plan = BatchQuery(jobs, **kw)
        plan.run()
        for j in jobs:
            single = _single(j, p=kw.get("p", 2.0), max_distance=kw.get("max_distance"), eps=kw.get("eps", 0.0))
            got = (j[3].cpu().numpy(), j[4].cpu().numpy())
            if "p" in kw:  # pow(): last-ulp differences are CUDA's own, identical in both calls
                np.testing.assert_array_equal(got[1], single[1])
            assert_bit_exact(got, single)


def test_batch_errors():
    import torch

    from kdtree import BatchQuery

    rng = np.random.default_rng(6)
    jobs, _ = _jobs(rng, SPECS[:3], torch)
    with pytest.raises(ValueError, match="k must be greater than zero"):
        t, dq = jobs[0][:2]
        n = dq.shape[0]
        BatchQuery([(t, dq, 0, torch.empty((n, 0), dtype=torch.float64, device="cuda"),
                     torch.empty((n, 0), dtype=torch.int64, device="cuda"))])
    with pytest.raises(ValueError):
        BatchQuery(jobs, p=0.5)
    jobs[1][1][3, 0] = float("nan")
    plan = BatchQuery(jobs)
    with pytest.raises(ValueError, match="finite"):
        plan.run()
    # the other jobs still ran
    assert_bit_exact((jobs[0][3].cpu().numpy(), jobs[0][4].cpu().numpy()), _single(jobs[0]))


@pytest.mark.parametrize("fixed", ["all", "none", None])
def test_small_k_jobs_as_packet_or_warp_tasks(oracle, monkeypatch, fixed):
    """Jobs of widths 2 and 3 with k <= 4 on large uniform trees run as packet
    tasks (32 sorted queries a warp: KD_BATCH_PACKET=all), as one query a warp
    (none), or as the first graph run's autotuner finds faster (unset: only
    widths with such jobs may be chosen); every job's results equal a lone call
    and the oracle in all three."""
    import torch

    from kdtree import BatchQuery

    if fixed is None:
        monkeypatch.delenv("KD_BATCH_PACKET", raising=False)
    else:
        monkeypatch.setenv("KD_BATCH_PACKET", fixed)
    rng = np.random.default_rng(31)
    specs = [(200_000, 3, 60_000, 1), (150_000, 3, 40_000, 4), (100_000, 2, 50_000, 2), (30_000, 8, 3000, 16),
             (120_000, 3, 20_000, 3)]
    jobs, host = _jobs(rng, specs, torch)
    plan = BatchQuery(jobs)
    plan.run(None)
    torch.cuda.synchronize()
    choice = plan.choice()
    if fixed == "all":
        assert choice["packet_widths"] == [2, 3], choice  # the 8-wide job has k = 16
    elif fixed == "none":
        assert choice["packet_widths"] == [], choice
    else:
        assert set(choice["packet_widths"]) <= {2, 3}, choice
    for job, (data, q) in zip(jobs, host):
        got = (job[3].cpu().numpy(), job[4].cpu().numpy())
        assert_bit_exact(got, _single(job))
    data, q = host[0]
    want = oracle.OracleKDTree(data, leafsize=jobs[0][0].leafsize).query(q[:2000], k=1, parallel=True)
    assert_bit_exact((jobs[0][3][:2000].cpu().numpy(), jobs[0][4][:2000].cpu().numpy()), want)
