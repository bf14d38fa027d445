"""Parity at the workloads' full sizes against the oracle.

- The N = 1,000,000 build (the plain-scale workload: uniform [0,1)^3 and the
  64-component Gaussian mixture, leafsize 16; and the precision workload's
  d = 16 and d = 64 scaled normal points) compared array by array, bit for bit:
  rows, indices, node records, split values, boxes (src/build.rs:345-359
  asserts the reference's own layouts identical).
- The precision workload (N = 1M, d in {16, 64}, per-dimension scale
  log-uniform in [0.1, 10], k = 32, L2): a slice of its 100,000 queries through
  the automatic path, the tensor-core filter and the warp traversal, bit for
  bit against the oracle."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bit_exact, gmm

pytestmark = pytest.mark.gpu


def _precision_data(d):
    rng = np.random.default_rng(300 + d)
    scale = np.exp(rng.uniform(np.log(0.1), np.log(10), d))
    data = rng.standard_normal((1_000_000, d)) * scale
    q = rng.standard_normal((100_000, d)) * scale
    return data, q


def _layout_equal(g, o):
    names = ("data", "indices", "node words", "split values", "boxes")
    for name, a, b in zip(names, g, o):
        assert a.shape == b.shape, name
        if a.dtype.kind == "f":
            same = a == b
            assert same.all(), f"{name}: {np.count_nonzero(~same)} of {a.size} differ"
        else:
            np.testing.assert_array_equal(a, b, err_msg=name)


@pytest.mark.parametrize("which", ["uniform-d3", "gmm-d3", "scaled-d16", "scaled-d64"])
def test_full_size_build_layout(oracle, which):
    from kdtree import KDTree

    if which == "uniform-d3":
        data = np.random.default_rng(2).uniform(size=(1_000_000, 3))
    elif which == "gmm-d3":
        data = gmm(1_000_000, 3, np.random.default_rng(4))
    else:
        data = _precision_data(int(which[-2:]))[0]
    g = KDTree(data, leafsize=16)._export()
    o = oracle.OracleKDTree(data, leafsize=16, parallel=True).export()
    _layout_equal(g, o)


@pytest.mark.parametrize("d", [16, 64])
def test_precision_workload_full_size(oracle, d):
    import torch

    from kdtree import KDTree, _core

    data, q = _precision_data(d)
    ns = 2000 if d == 16 else 600
    rng = np.random.default_rng(d)
    pick = np.sort(rng.choice(q.shape[0], ns, replace=False))
    qs = q[pick]
    want = oracle.OracleKDTree(data, leafsize=16, parallel=True).query(qs, k=32, parallel=True)
    tree = KDTree(data, leafsize=16)
    assert_bit_exact(tree.query(qs, k=32), want)
    L = _core._lib
    P, u64, dd = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    L.kd_query_device_path.argtypes = [P, P, u64, u64, dd, ctypes.c_int, dd, dd, P, P, P, ctypes.c_int, P]
    L.kd_query_device_path.restype = ctypes.c_int
    dq = torch.from_numpy(qs).cuda()
    for path in (3, 4):  # tensor-core filter, warp traversal
        od = torch.empty((ns, 32), dtype=torch.float64, device="cuda")
        oi = torch.empty((ns, 32), dtype=torch.int64, device="cuda")
        st = L.kd_query_device_path(tree._h, P(dq.data_ptr()), dq.numel(), 32, 2.0, 0, 0.0, 0.0, P(od.data_ptr()),
                                    P(oi.data_ptr()), None, path, None)
        assert st == 0, _core._last_error()
        assert_bit_exact((od.cpu().numpy(), oi.cpu().numpy()), want)
