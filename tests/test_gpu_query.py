"""GPU query against the oracle, bit for bit: every metric and strategy
(Packed d<=8 with the d4 / d8 chunk orders, Folded 9..16, Streamed), k from 1
to 32, eps > 0 (DFS-order dependent), max_distance padding, queries outside the
root box (seeded CellBound), clustered data (order_by_box descents), and the
plain workloads at full size."""
import numpy as np
import pytest

from helpers import assert_bit_exact, assert_lp_close, gmm

pytestmark = pytest.mark.gpu


def _both(oracle, data, queries, leafsize, **kw):
    from kdtree import KDTree

    g = KDTree(data, leafsize=leafsize).query(queries, **kw)
    o = oracle.OracleKDTree(data, leafsize=leafsize).query(queries, parallel=True, **kw)
    return g, o


@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 6, 7, 8, 9, 12, 16, 17, 24, 64])
@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
def test_widths_and_metrics(oracle, d, p):
    rng = np.random.default_rng(100 * d + int(p if np.isfinite(p) else 99))
    data = rng.normal(size=(3000, d))
    q = rng.normal(size=(300, d)) * 1.3  # some queries outside the root box
    for k in (1, 5, 16):
        g, o = _both(oracle, data, q, 6, k=k, p=p)
        assert_bit_exact(g, o)


@pytest.mark.parametrize("k", [1, 2, 3, 4, 7, 8, 9, 15, 16, 17, 31, 32])
def test_k_values(oracle, k):
    rng = np.random.default_rng(k)
    data = rng.uniform(size=(20_000, 3))
    q = rng.uniform(size=(2000, 3))
    assert_bit_exact(*_both(oracle, data, q, 16, k=k))


@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
@pytest.mark.parametrize("eps", [0.1, 1.0])
def test_eps_follows_reference_dfs_order(oracle, p, eps):
    rng = np.random.default_rng(7)
    data = gmm(30_000, 3, rng)
    q = gmm(1000, 3, rng)
    assert_bit_exact(*_both(oracle, data, q, 16, k=8, p=p, eps=eps))


@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
def test_max_distance(oracle, p):
    rng = np.random.default_rng(11)
    data = rng.uniform(size=(20_000, 3))
    q = rng.uniform(size=(1000, 3)) * 1.2
    for md in (0.0, 0.01, 0.05):
        assert_bit_exact(*_both(oracle, data, q, 16, k=16, p=p, max_distance=md))


def test_general_p(oracle):
    """L^p distances go through pow(): CUDA's and libm's differ in the last
    places, so distances are compared within lp_max_ulps(d, p) ulp (the bound
    is derived in tests/helpers.py) and indices exactly."""
    rng = np.random.default_rng(13)
    data = rng.normal(size=(5000, 4))
    q = rng.normal(size=(500, 4))
    for p in (1.5, 3.0):
        g, o = _both(oracle, data, q, 8, k=6, p=p)
        assert_lp_close(g, o, 4, p)


def test_ties(oracle):
    rng = np.random.default_rng(5)
    data = rng.integers(0, 5, size=(20_000, 3)).astype(float)
    q = rng.integers(0, 5, size=(500, 3)).astype(float)
    for p in (1.0, 2.0, np.inf):
        assert_bit_exact(*_both(oracle, data, q, 4, k=9, p=p))


def test_single_query_shape(oracle):
    from kdtree import KDTree

    data = np.random.default_rng(1).normal(size=(100, 3))
    d, i = KDTree(data).query(data[7], k=3)
    assert d.shape == (3,) and i.shape == (3,) and i[0] == 7 and d[0] == 0.0


def test_k_greater_than_points(oracle):
    data = np.random.default_rng(1).normal(size=(5, 2))
    g, o = _both(oracle, data, data[:3], 32, k=9)
    assert_bit_exact(g, o)
    assert (g[1][:, 5:] == 5).all() and np.isinf(g[0][:, 5:]).all()


@pytest.mark.parametrize("dist", ["uniform", "gmm"])
@pytest.mark.parametrize("k", [1, 16])
@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
def test_plain_scale_sampled(oracle, dist, k, p):
    """N=1,000,000, d=3, leafsize 16 (data seed 2), 1,000,000 queries (seed 3):
    all of them on the GPU; a 20,000-query sample bit-exact against the oracle,
    and every result sorted, in range, and consistent with its own distances."""
    from kdtree import KDTree

    rd, rq = np.random.default_rng(2), np.random.default_rng(3)
    if dist == "uniform":
        data, q = rd.uniform(size=(1_000_000, 3)), rq.uniform(size=(1_000_000, 3))
    else:
        centres = np.random.default_rng(4).uniform(size=(64, 3))
        data = centres[rd.integers(0, 64, 1_000_000)] + 0.01 * rd.standard_normal((1_000_000, 3))
        q = centres[rq.integers(0, 64, 1_000_000)] + 0.01 * rq.standard_normal((1_000_000, 3))
    t = KDTree(data, leafsize=16)
    gd, gi = t.query(q, k=k, p=p)
    assert np.all(np.diff(gd, axis=1) >= 0)
    assert gi.min() >= 0 and gi.max() < 1_000_000
    diff = np.abs(data[gi[:, 0]] - q)
    ref0 = diff.max(1) if np.isinf(p) else (diff.sum(1) if p == 1 else np.sqrt((diff**2).sum(1)))
    np.testing.assert_allclose(gd[:, 0], ref0, rtol=1e-12, atol=1e-15)
    sel = np.random.default_rng(9).choice(1_000_000, 20_000, replace=False)
    o = oracle.OracleKDTree(data, leafsize=16).query(q[sel], k=k, p=p, parallel=True)
    assert_bit_exact((gd[sel], gi[sel]), o)


@pytest.mark.parametrize("d,p", [(3, 2.0), (5, 1.0), (8, np.inf), (17, 2.0)])
@pytest.mark.parametrize("k", [33, 64, 150])
def test_large_k(oracle, d, p, k):
    """k beyond the register lists: the list lives in the query's output row."""
    rng = np.random.default_rng(k + d)
    data = rng.normal(size=(4000, d))
    q = rng.normal(size=(300, d))
    assert_bit_exact(*_both(oracle, data, q, 16, k=k, p=p))


def test_k_far_beyond_n(oracle):
    data = np.random.default_rng(3).normal(size=(40, 3))
    g, o = _both(oracle, data, data[:10] + 0.01, 8, k=100)
    assert_bit_exact(g, o)
    assert (g[1][:, 40:] == 40).all()


@pytest.mark.parametrize("k", [1, 16, 40])
def test_host_buffers_pinned_and_pageable(oracle, k):
    """kd_query with page-locked outputs (kernels write them directly) and with
    pageable ones (device staging + download): identical results."""
    import ctypes

    import torch

    from kdtree import KDTree, _core

    rng = np.random.default_rng(40 + k)
    data = rng.uniform(size=(50_000, 3))
    q = rng.uniform(size=(30_000, 3))
    t = KDTree(data, leafsize=16)
    L = _core._lib
    P = ctypes.c_void_p
    outs = []
    for pinned in (True, False):
        hq = torch.from_numpy(q)
        hd = torch.empty((len(q), k), dtype=torch.float64)
        hi = torch.empty((len(q), k), dtype=torch.int64)
        if pinned:
            hq, hd, hi = hq.pin_memory(), hd.pin_memory(), hi.pin_memory()
        st = L.kd_query(t._h, P(hq.data_ptr()), hq.numel(), k, 2.0, 0, 0.0, 0.0, 0, P(hd.data_ptr()),
                        P(hi.data_ptr()))
        assert st == 0, _core._last_error()
        outs.append((hd.numpy().copy(), hi.numpy().copy()))
    assert_bit_exact(outs[0], outs[1])
    o = oracle.OracleKDTree(data, leafsize=16).query(q[:3000], k=k, parallel=True)
    assert_bit_exact((outs[0][0][:3000], outs[0][1][:3000]), o)


def test_result_arrays_come_from_the_page_locked_pool(oracle):
    """KDTree.query returns ordinary numpy arrays backed by page-locked blocks
    (kd_host_alloc), which the kernel writes directly; a block freed with its
    arrays is handed out again, and results stay valid after the tree is gone."""
    import ctypes
    import gc

    from kdtree import KDTree, _core

    rng = np.random.default_rng(21)
    data = rng.uniform(size=(50_000, 3))
    q = rng.uniform(size=(20_000, 3))
    tree = KDTree(data, leafsize=16)
    want = oracle.OracleKDTree(data, leafsize=16).query(q, k=8, parallel=True)
    d1, i1 = tree.query(q, k=8)
    assert_bit_exact((d1, i1), want)
    assert d1.flags.c_contiguous and d1.dtype == np.float64 and i1.dtype == np.int64
    addrs = {d1.ctypes.data, i1.ctypes.data}
    del d1, i1
    gc.collect()  # numpy's comparison helpers can leave the arrays in a reference cycle
    L = _core._lib
    p = ctypes.c_void_p()
    assert L.kd_host_alloc(20_000 * 8 * 8, ctypes.byref(p)) == 0 and p.value in addrs  # a freed block comes back
    L.kd_host_free(p)
    d2, i2 = tree.query(q, k=8)
    assert {d2.ctypes.data, i2.ctypes.data} == addrs
    del tree
    assert_bit_exact((d2, i2), want)
    assert L.kd_host_alloc(1 << 20, ctypes.byref(p)) == 0 and p.value
    q_ = ctypes.c_void_p(p.value)
    L.kd_host_free(p)
    assert L.kd_host_alloc(1 << 20, ctypes.byref(p)) == 0 and p.value == q_.value
    L.kd_host_free(p)
    L.kd_host_free(None)
