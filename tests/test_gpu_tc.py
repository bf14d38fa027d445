"""The tensor-core filter path (L2, eps = 0, 16 <= d <= 128, k <= 32) against
the oracle, bit for bit, and against the engine's reference-order FP64 path.

It scores every (query, point) pair with BF16 tcgen05 MMAs and uses the score
only to reject pairs whose exact distance provably exceeds the current bound;
survivors are ranked by the reference's exact FP64 distance (Folded order at
d <= 16, Streamed above), so results must match the oracle exactly."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bit_exact

pytestmark = pytest.mark.gpu

PATH_REFERENCE_ORDER, PATH_TENSOR_CORE = 1, 3


def scaled_normal(rng, n, d, scale):
    return rng.standard_normal((n, d)) * scale


def _path_query(tree, q, k, path, max_distance=None):
    import torch

    from kdtree import _core

    L = _core._lib
    P, u64, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    L.kd_query_device_path.argtypes = [P, P, u64, u64, dbl, ctypes.c_int, dbl, dbl, P, P, P, ctypes.c_int, P]
    L.kd_query_device_path.restype = ctypes.c_int
    dq = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    od = torch.empty((q.shape[0], k), dtype=torch.float64, device="cuda")
    oi = torch.empty((q.shape[0], k), dtype=torch.int64, device="cuda")
    surv = torch.zeros(3, dtype=torch.int64, device="cuda")  # filter survivors, near ties, full reruns
    st = L.kd_query_device_path(tree._h, P(dq.data_ptr()), dq.numel(), k, 2.0, int(max_distance is not None),
                                float(max_distance or 0.0), 0.0, P(od.data_ptr()), P(oi.data_ptr()), None, path,
                                P(surv.data_ptr()))
    assert st == 0, _core._last_error()
    return od.cpu().numpy(), oi.cpu().numpy(), int(surv[0].item())


@pytest.mark.parametrize("d", [16, 17, 31, 64, 100, 128])
@pytest.mark.parametrize("k", [1, 5, 32])
def test_tc_matches_oracle(oracle, d, k):
    from kdtree import KDTree

    rng = np.random.default_rng(1000 + 7 * d + k)
    scale = np.exp(rng.uniform(np.log(0.1), np.log(10), d))
    data = scaled_normal(rng, 20_000, d, scale)
    q = scaled_normal(rng, 1000, d, scale)
    t = KDTree(data, leafsize=16)
    g = t.query(q, k=k)  # the automatic choice is the tensor-core path here
    o = oracle.OracleKDTree(data, leafsize=16).query(q, k=k, parallel=True)
    assert_bit_exact(g, o)
    d_tc, i_tc, surv = _path_query(t, q, k, PATH_TENSOR_CORE)
    assert_bit_exact((d_tc, i_tc), o)
    assert 0 < surv < 0.05 * q.shape[0] * data.shape[0]


@pytest.mark.parametrize("d", [16, 64])
def test_tc_agrees_with_reference_order(oracle, d):
    from kdtree import KDTree

    rng = np.random.default_rng(d)
    data = rng.standard_normal((30_000, d))
    q = rng.standard_normal((500, d))
    t = KDTree(data, leafsize=32)
    a = _path_query(t, q, 32, PATH_TENSOR_CORE)
    b = _path_query(t, q, 32, PATH_REFERENCE_ORDER)
    assert_bit_exact(a[:2], b[:2])


def test_tc_max_distance_padding(oracle):
    from kdtree import KDTree

    rng = np.random.default_rng(5)
    data = rng.standard_normal((20_000, 24))
    q = rng.standard_normal((700, 24))
    for md in (0.0, 4.0, 5.5):
        g = KDTree(data, leafsize=16).query(q, k=16, max_distance=md)
        o = oracle.OracleKDTree(data, leafsize=16).query(q, k=16, max_distance=md, parallel=True)
        assert_bit_exact(g, o)


def test_tc_ties_and_duplicates(oracle):
    from kdtree import KDTree

    rng = np.random.default_rng(9)
    data = rng.integers(0, 3, size=(12_000, 16)).astype(float)
    q = rng.integers(0, 3, size=(400, 16)).astype(float)
    g = KDTree(data, leafsize=8).query(q, k=20)
    o = oracle.OracleKDTree(data, leafsize=8).query(q, k=20, parallel=True)
    assert_bit_exact(g, o)


def test_tc_ragged_sizes(oracle):
    """Point and query counts that fill no tile exactly, N < k, far queries."""
    from kdtree import KDTree

    rng = np.random.default_rng(11)
    for n, nq in ((1, 3), (20, 130), (257, 129), (1000, 1)):
        data = rng.standard_normal((n, 20))
        q = rng.standard_normal((nq, 20)) * 3
        g = KDTree(data, leafsize=4).query(q, k=32)
        o = oracle.OracleKDTree(data, leafsize=4).query(q, k=32, parallel=True)
        assert_bit_exact(g, o)


def test_tc_precision_workload_sampled(oracle):
    """d=64 scaled normal (per-dimension scale log-uniform in [0.1, 10]),
    N=200,000, k=32: 2,000 queries on the tensor-core path, bit-exact."""
    from kdtree import KDTree

    rng = np.random.default_rng(64)
    scale = np.exp(rng.uniform(np.log(0.1), np.log(10), 64))
    data = scaled_normal(rng, 200_000, 64, scale)
    q = scaled_normal(rng, 2000, 64, scale)
    g = KDTree(data, leafsize=16).query(q, k=32)
    o = oracle.OracleKDTree(data, leafsize=16).query(q, k=32, parallel=True)
    assert_bit_exact(g, o)
