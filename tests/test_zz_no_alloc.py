"""kd_query_device_noalloc against kd_query_device, through the C ABI.

The allocation-free entry point serves callers that cannot let a library
allocate device memory (a framework holding nearly all of HBM in its own pool,
or a latency-bound request loop).  Its status word and per-query scratch live in
one fixed device array shared by every call, so these checks call it twice in a
row, with different queries, and require each result to equal the allocating
entry point's bit for bit (the tolerance every other FP64 parity test here
uses).  This file is collected last so a failure here comes after every other
test has run; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_VALUES = 524256  # KD_NOALLOC_MAX_VALUES in include/kdtree_gb300.h


def _lib():
    from kdtree import _core

    L = _core._lib
    P = ctypes.c_void_p
    u64 = ctypes.c_uint64
    d = ctypes.c_double
    L.kd_query_device_noalloc.argtypes = [P, P, u64, u64, d, ctypes.c_int, d, d, P, P, P]
    L.kd_query_device_noalloc.restype = ctypes.c_int
    return L, _core


def _call(fn, tree, dq, k, p, has_max, max_distance, eps, stream):
    import torch

    nq = dq.shape[0]
    out_d = torch.full((nq, k), -1.0, dtype=torch.float64, device=dq.device)
    out_i = torch.full((nq, k), -1, dtype=torch.int64, device=dq.device)
    st = fn(tree._h, ctypes.c_void_p(dq.data_ptr()), dq.numel(), k, p, has_max, max_distance, eps,
            ctypes.c_void_p(out_d.data_ptr()), ctypes.c_void_p(out_i.data_ptr()), ctypes.c_void_p(stream))
    return st, out_d.cpu().numpy(), out_i.cpu().numpy()


@pytest.mark.parametrize(
    "d,k,p,max_distance,n_points",
    [
        (3, 16, 2.0, None, 50_000),     # register path: only the status word is scratch
        (5, 8, 1.0, None, 50_000),      # dynamic width: CellBound axes live in the scratch
        (20, 4, np.inf, 1.5, 50_000),   # Streamed L-inf with padding
        (64, 8, 2.0, None, 20_000),     # kd_query_device takes the tensor-core filter here
    ],
)
def test_noalloc_matches_allocating_entry_point(d, k, p, max_distance, n_points):
    import torch

    from kdtree import KDTree

    L, core = _lib()
    rng = np.random.default_rng(100 + d)
    data = rng.normal(size=(n_points, d))
    tree = KDTree(data, leafsize=16)
    stream = torch.cuda.Stream()
    nq = MAX_VALUES // d
    has_max = max_distance is not None
    md = float(max_distance) if has_max else 0.0
    P = ctypes.c_void_p
    # two query sets; the allocating entry point's answers first
    sets = []
    for call in range(2):
        q = rng.normal(size=(nq - 17 * call, d)) * 1.2
        dq = torch.from_numpy(q).cuda()
        st_ref, ref_d, ref_i = _call(L.kd_query_device, tree, dq, k, p, int(has_max), md, 0.0, stream.cuda_stream)
        assert st_ref == 0, core._last_error()
        out_d = torch.full((dq.shape[0], k), -1.0, dtype=torch.float64, device="cuda")
        out_i = torch.full((dq.shape[0], k), -1, dtype=torch.int64, device="cuda")
        sets.append((dq, ref_d, ref_i, out_d, out_i))
    torch.cuda.synchronize()
    free_before = None
    for call, (dq, ref_d, ref_i, out_d, out_i) in enumerate(sets):  # two calls in a row share the scratch
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        st = L.kd_query_device_noalloc(tree._h, P(dq.data_ptr()), dq.numel(), k, p, int(has_max), md, 0.0,
                                       P(out_d.data_ptr()), P(out_i.data_ptr()), P(stream.cuda_stream))
        assert st == 0, core._last_error()
        torch.cuda.synchronize()
        if call == 1:
            # the second call maps no device memory (its kernels were loaded by the first)
            assert torch.cuda.mem_get_info()[0] == free_before
        got_d, got_i = out_d.cpu().numpy(), out_i.cpu().numpy()
        np.testing.assert_array_equal(got_i, ref_i)
        assert np.array_equal(got_d, ref_d), "distances differ from kd_query_device"


def test_noalloc_rejects_oversized_batch_and_bad_queries():
    import torch

    from kdtree import KDTree

    L, core = _lib()
    tree = KDTree(np.random.default_rng(1).normal(size=(1000, 3)), leafsize=16)
    big = torch.zeros((MAX_VALUES // 3 + 1, 3), dtype=torch.float64, device="cuda")
    st, _, _ = _call(L.kd_query_device_noalloc, tree, big, 4, 2.0, 0, 0.0, 0.0, 0)
    assert st == 102 and "at most 524256" in core._last_error()
    bad = torch.zeros((10, 3), dtype=torch.float64, device="cuda")
    bad[3, 1] = float("nan")
    st, _, _ = _call(L.kd_query_device_noalloc, tree, bad, 4, 2.0, 0, 0.0, 0.0, 0)
    assert st == 7 and core._last_error() == "all coordinates must be finite"
    # the status word left set by that call must not leak into the next one
    good = torch.zeros((10, 3), dtype=torch.float64, device="cuda")
    st, _, got_i = _call(L.kd_query_device_noalloc, tree, good, 4, 2.0, 0, 0.0, 0.0, 0)
    assert st == 0
    st, _, ref_i = _call(L.kd_query_device, tree, good, 4, 2.0, 0, 0.0, 0.0, 0)
    np.testing.assert_array_equal(got_i, ref_i)
