"""The automatic choice between the two eps = 0 traversals where neither is
clearly ahead (widths 2 and 3, 32,768 to 524,287 queries): the first automatic
call of each class on a tree runs both on its batch and keeps the faster.
Every call's results equal the explicit paths' and the oracle's, and the
timed call's near-tie counters count one run (the packet traversal's)."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bit_exact

pytestmark = pytest.mark.gpu

PATH_AUTO, PATH_PACKET, PATH_WARP = 0, 2, 4


def _lib():
    from kdtree import _core

    L = _core._lib
    P, u64, d = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    L.kd_query_device_path.argtypes = [P, P, u64, u64, d, ctypes.c_int, d, d, P, P, P, ctypes.c_int, P]
    L.kd_query_device_path.restype = ctypes.c_int
    return L, _core


@pytest.mark.parametrize("d,k,nq", [(3, 8, 40_000), (2, 24, 150_000)])
def test_timed_choice_matches_explicit_paths(oracle, d, k, nq):
    import torch

    from kdtree import KDTree

    L, core = _lib()
    rng = np.random.default_rng(50 + d + k)
    data = rng.uniform(size=(200_000, d))
    q = rng.uniform(size=(nq, d)) * 1.1 - 0.05
    tree = KDTree(data, leafsize=16)
    dq = torch.from_numpy(q).cuda()
    P = ctypes.c_void_p

    def call(path):
        od = torch.full((nq, k), -1.0, dtype=torch.float64, device="cuda")
        oi = torch.full((nq, k), -1, dtype=torch.int64, device="cuda")
        cnt = torch.zeros(3, dtype=torch.int64, device="cuda")  # survivors, near ties, full reruns
        st = L.kd_query_device_path(tree._h, P(dq.data_ptr()), dq.numel(), k, 2.0, 0, 0.0, 0.0,
                                    P(od.data_ptr()), P(oi.data_ptr()), None, path, P(cnt.data_ptr()))
        assert st == 0, core._last_error()
        return od.cpu().numpy(), oi.cpu().numpy(), tuple(int(x) for x in cnt.cpu())

    first = call(PATH_AUTO)  # runs both traversals, keeps the faster
    second = call(PATH_AUTO)  # the kept one
    warp = call(PATH_WARP)
    packet = call(PATH_PACKET)
    for got in (first, second, packet):
        assert_bit_exact(got[:2], warp[:2])
    assert first[2] == packet[2]
    assert second[2] in (warp[2], packet[2])
    want = oracle.OracleKDTree(data, leafsize=16).query(q[:2000], k=k, parallel=True)
    assert_bit_exact((first[0][:2000], first[1][:2000]), want)
