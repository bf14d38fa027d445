"""The warp-per-query kernels at every width they take (1..128): the best-first
traversal (eps = 0; compile-time widths 1, 2, 3, 4, 8, 16, the runtime-width
kernel with padded FP32 rows for the rest) and the reference-order warp
kernel (any eps, general p), each bit for bit against the oracle, with k up
to 64 (two list slots per lane above 32), queries outside the root box
(seeded CellBound), clustered data (order_by_box nodes) and Packed d4 / d8
chunk orders (leaves of odd lengths)."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bit_exact, assert_lp_close, gmm

pytestmark = pytest.mark.gpu

WIDTHS = list(range(1, 21)) + [24, 31, 32, 33, 48, 63, 64, 100, 128]


def _path(tree, q, k, p, path, eps=0.0, max_distance=None):
    import torch

    from kdtree import _core

    L = _core._lib
    P, u64, d = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    L.kd_query_device_path.argtypes = [P, P, u64, u64, d, ctypes.c_int, d, d, P, P, P, ctypes.c_int, P]
    L.kd_query_device_path.restype = ctypes.c_int
    dq = torch.from_numpy(q).cuda()
    od = torch.full((q.shape[0], k), -1.0, dtype=torch.float64, device="cuda")
    oi = torch.full((q.shape[0], k), -1, dtype=torch.int64, device="cuda")
    st = L.kd_query_device_path(tree._h, P(dq.data_ptr()), dq.numel(), k, p, int(max_distance is not None),
                                float(max_distance or 0.0), eps, P(od.data_ptr()), P(oi.data_ptr()), None, path, None)
    assert st == 0, _core._last_error()
    return od.cpu().numpy(), oi.cpu().numpy()


@pytest.mark.parametrize("d", WIDTHS)
@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
def test_warp_and_reference_order_paths(oracle, d, p):
    from kdtree import KDTree

    rng = np.random.default_rng(1000 + 7 * d + int(p if np.isfinite(p) else 5))
    n = 4000 if d <= 32 else 2500
    data = gmm(n, d, rng, components=8, sigma=0.05) if d % 3 == 0 else rng.normal(size=(n, d))
    q = (data[rng.integers(0, n, 150)] + 0.05 * rng.normal(size=(150, d))) * 1.15
    leaf = int(rng.choice([5, 7, 16]))
    tree = KDTree(data, leafsize=leaf)
    ot = oracle.OracleKDTree(data, leafsize=leaf)
    for k in (1, 7, 33, 64):
        want = ot.query(q, k=k, p=p, parallel=True)
        assert_bit_exact(_path(tree, q, k, p, 4), want)  # best-first warp
        assert_bit_exact(_path(tree, q, k, p, 1), want)  # reference order, one warp a query


@pytest.mark.parametrize("d", [1, 3, 5, 8, 13, 16, 20, 64])
@pytest.mark.parametrize("p", [1.0, 2.0, 3.0, np.inf])
def test_eps_and_general_p_in_reference_order(oracle, d, p):
    """eps > 0 and L^p run the reference-order warp kernel; the result depends
    on its visiting order, which must be the reference's."""
    from kdtree import KDTree

    rng = np.random.default_rng(2000 + d)
    data = gmm(5000, d, rng, components=16, sigma=0.03)
    q = gmm(200, d, rng, components=16, sigma=0.03)
    tree = KDTree(data, leafsize=8)
    ot = oracle.OracleKDTree(data, leafsize=8)
    for eps, k in ((0.0, 5), (0.5, 5), (2.0, 12)):
        got = tree.query(q, k=k, p=p, eps=eps)
        want = ot.query(q, k=k, p=p, eps=eps, parallel=True)
        if p == 3.0:  # pow(): CUDA and libm differ in the last places (tests/helpers.py)
            assert_lp_close(got, want, d, p)
        else:
            assert_bit_exact(got, want)


@pytest.mark.parametrize("d", [4, 8])
def test_packed_chunk_orders_in_warp_kernels(oracle, d):
    """Packed d4 pairs / d8 groups of 8 use their pairwise summation order only
    inside full chunks of a leaf (kernel.rs:517-562): odd leaf lengths put
    points in both parts."""
    from kdtree import KDTree

    rng = np.random.default_rng(40 + d)
    data = rng.uniform(size=(30_001, d)).round(3)  # many near-equal sums
    q = rng.uniform(size=(2000, d)).round(3)
    for leaf in (7, 9, 13):
        tree = KDTree(data, leafsize=leaf)
        ot = oracle.OracleKDTree(data, leafsize=leaf)
        for p in (1.0, 2.0):
            want = ot.query(q, k=9, p=p, parallel=True)
            assert_bit_exact(_path(tree, q, 9, p, 4), want)
            assert_bit_exact(_path(tree, q, 9, p, 1), want)
            assert_bit_exact(tree.query(q, k=9, p=p), want)
