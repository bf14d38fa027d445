"""kd_query_async: the stream-ordered query (no host wait) gives exactly
kd_query_device's results, leaves its error status in device memory, and
returns while its stream is still busy."""
import ctypes

import numpy as np
import pytest

from helpers import assert_bit_exact

pytestmark = pytest.mark.gpu


def _sync_query(tree, dq, k, p, eps=0.0):
    import torch

    from kdtree import _core

    od = torch.empty((dq.shape[0], k), dtype=torch.float64, device="cuda")
    oi = torch.empty((dq.shape[0], k), dtype=torch.int64, device="cuda")
    P = ctypes.c_void_p
    st = _core._lib.kd_query_device(tree._h, P(dq.data_ptr()), dq.numel(), k, p, 0, 0.0, eps, P(od.data_ptr()),
                                    P(oi.data_ptr()), None)
    assert st == 0, _core._last_error()
    return od.cpu().numpy(), oi.cpu().numpy()


@pytest.mark.parametrize("d,k,p,eps", [(3, 16, 2.0, 0.0), (8, 5, 1.0, 0.0), (16, 32, 2.0, 0.0),
                                       (64, 8, 2.0, 0.0), (5, 4, np.inf, 0.3), (3, 3, 3.0, 0.0)])
def test_async_equals_device_call(d, k, p, eps):
    import torch

    from kdtree import KDTree

    rng = np.random.default_rng(900 + d)
    data = rng.normal(size=(40_000, d))
    tree = KDTree(data, leafsize=16)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    batches = [torch.from_numpy(rng.normal(size=(6000 + 17 * i, d))).cuda() for i in range(4)]
    outs = []
    for i, dq in enumerate(batches):  # four calls in flight on two streams
        od = torch.empty((dq.shape[0], k), dtype=torch.float64, device="cuda")
        oi = torch.empty((dq.shape[0], k), dtype=torch.int64, device="cuda")
        status = torch.full((1,), 7, dtype=torch.int32, device="cuda")
        outs.append((od, oi, status))
    torch.cuda.synchronize()  # the buffers' own fills (default stream) are done before the calls' streams start
    for i, (dq, (od, oi, status)) in enumerate(zip(batches, outs)):
        tree.query_async(dq, od, oi, status, k=k, p=p, eps=eps, stream=streams[i % 2])
    torch.cuda.synchronize()
    for dq, (od, oi, status) in zip(batches, outs):
        assert int(status.item()) == 0
        got = (od.cpu().numpy(), oi.cpu().numpy())
        want = _sync_query(tree, dq, k, p, eps)
        if p == 3.0:
            np.testing.assert_array_equal(got[1], want[1])
            assert np.array_equal(got[0], want[0])  # same device, same pow()
        else:
            assert_bit_exact(got, want)


def test_async_returns_before_the_stream_is_done():
    import torch

    from kdtree import KDTree

    rng = np.random.default_rng(3)
    tree = KDTree(rng.uniform(size=(100_000, 3)), leafsize=16)
    dq = torch.from_numpy(rng.uniform(size=(50_000, 3))).cuda()
    od = torch.empty((50_000, 16), dtype=torch.float64, device="cuda")
    oi = torch.empty((50_000, 16), dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    tree.query_async(dq, od, oi, status, k=16, stream=stream)  # warm: pool, kernels loaded
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        torch.cuda._sleep(1_000_000_000)  # about half a second of GPU time ahead of the query
    tree.query_async(dq, od, oi, status, k=16, stream=stream)
    assert not stream.query(), "kd_query_async waited for its stream"
    stream.synchronize()
    assert int(status.item()) == 0
    assert_bit_exact((od.cpu().numpy(), oi.cpu().numpy()), _sync_query(tree, dq, 16, 2.0))


def test_async_errors():
    import torch

    from kdtree import KDTree

    rng = np.random.default_rng(4)
    tree = KDTree(rng.uniform(size=(1000, 3)), leafsize=16)
    dq = torch.from_numpy(rng.uniform(size=(100, 3))).cuda()
    dq[7, 2] = float("nan")
    od = torch.empty((100, 4), dtype=torch.float64, device="cuda")
    oi = torch.empty((100, 4), dtype=torch.int64, device="cuda")
    status = torch.full((1,), 12345, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    tree.query_async(dq, od, oi, status, k=4)  # accepted: the non-finite query shows in the status
    torch.cuda.synchronize()
    assert int(status.item()) & 1
    # a scalar error raises at once; the finiteness check still lands in the status
    status.fill_(0)
    torch.cuda.synchronize()
    with pytest.raises(ValueError, match="p must be finite"):
        tree.query_async(dq, od, oi, status, k=4, p=0.5)
    torch.cuda.synchronize()
    assert int(status.item()) & 1
    with pytest.raises(ValueError, match="k must be greater than zero"):
        tree.query_async(dq, od, oi, status, k=0)
