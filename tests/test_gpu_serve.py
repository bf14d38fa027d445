"""The serving loop (kd_server_*): requests of many sizes, widths and k,
submitted concurrently and batched together, each get exactly what a lone
KDTree.query call returns (bit for bit); a bad request fails alone."""
import threading

import numpy as np
import pytest

from helpers import assert_bit_exact, gmm

pytestmark = pytest.mark.gpu


def _trees(rng):
    from kdtree import KDTree

    out = []
    for n, d in ((60_000, 3), (20_000, 8), (30_000, 16), (5000, 5), (80_000, 2), (10_000, 3)):
        out.append((KDTree(gmm(n, d, rng), leafsize=int(rng.choice([16, 32]))), d))
    return out


@pytest.mark.parametrize("max_batch", [0, 3000])
def test_mixed_requests_match_lone_queries(max_batch):
    from kdtree import Server

    rng = np.random.default_rng(50 + max_batch)
    trees = _trees(rng)
    srv = Server([t for t, _ in trees], max_batch_queries=max_batch)
    reqs = []
    for _ in range(120):
        ti = int(rng.integers(len(trees)))
        nq = int(np.exp(rng.uniform(0, np.log(3000))))
        k = int(np.exp(rng.uniform(0, np.log(64))).round())
        q = gmm(nq, trees[ti][1], rng)
        reqs.append((ti, q, k))
    tickets = [None] * len(reqs)

    def submit(lo, hi):
        for i in range(lo, hi):
            ti, q, k = reqs[i]
            tickets[i] = srv.submit(ti, q, k)

    threads = [threading.Thread(target=submit, args=(i, min(i + 30, len(reqs)))) for i in range(0, len(reqs), 30)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for (ti, q, k), tk in zip(reqs, tickets):
        d, i, lat = srv.wait(tk)
        assert lat > 0
        assert_bit_exact((d, i), trees[ti][0].query(q, k=k))
    srv.close()


def test_bad_request_fails_alone():
    from kdtree import Server

    rng = np.random.default_rng(4)
    trees = _trees(rng)[:2]
    srv = Server([t for t, _ in trees], max_batch_queries=4096)
    good = gmm(500, 3, rng)
    bad = gmm(300, 3, rng)
    bad[7, 1] = np.nan
    t_good = srv.submit(0, good, 8)
    t_bad = srv.submit(0, bad, 8)
    t_good2 = srv.submit(1, gmm(100, 8, rng), 3)
    assert_bit_exact(srv.wait(t_good)[:2], trees[0][0].query(good, k=8))
    with pytest.raises(ValueError, match="finite"):
        srv.wait(t_bad)
    srv.wait(t_good2)
    with pytest.raises(ValueError, match="k must be greater than zero"):
        srv.submit(0, good, 0)
    big = gmm(5000, 3, rng)  # larger than one batch: runs as two pieces
    assert_bit_exact(srv.wait(srv.submit(0, big, 4))[:2], trees[0][0].query(big, k=4))
    with pytest.raises(RuntimeError, match="capacity"):  # one query's results exceed a batch
        srv.submit(0, good[:1], 300_000)
    with pytest.raises(ValueError, match="dimension mismatch"):
        srv.submit(1, good, 4)
    srv.close()


def test_large_requests_run_in_pieces_beside_small_ones():
    """Requests above the piece size (about 4 ms of the tree's estimated GPU
    time, at most 16,384 queries) run as several pieces that small requests
    overtake; each result still equals a lone query, and a non-finite query in
    any piece fails the whole request."""
    from kdtree import Server

    rng = np.random.default_rng(77)
    trees = _trees(rng)
    srv = Server([t for t, _ in trees])
    big = gmm(40_000, 3, rng)
    bad_big = gmm(35_000, 8, rng)
    bad_big[30_000, 2] = np.inf  # in its second piece
    t_big = srv.submit(0, big, 16)
    t_bad = srv.submit(1, bad_big, 4)
    small = [(int(rng.integers(len(trees))), int(rng.integers(1, 500)), int(rng.integers(1, 30))) for _ in range(40)]
    smalls = []
    for ti, nq, k in small:
        q = gmm(nq, trees[ti][1], rng)
        smalls.append((ti, q, k, srv.submit(ti, q, k)))
    for ti, q, k, tk in smalls:
        assert_bit_exact(srv.wait(tk)[:2], trees[ti][0].query(q, k=k))
    d, i, lat = srv.wait(t_big)
    assert_bit_exact((d, i), trees[0][0].query(big, k=16))
    with pytest.raises(ValueError, match="finite"):
        srv.wait(t_bad)
    srv.close()
