"""Both query kernels for compile-time widths agree with the oracle bit for bit:
the packet traversal (the default for eps = 0) and the reference-order descent
(used for eps > 0, forced here with KD_QUERY_MODE=dfs in a child process)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import assert_bit_exact, gmm

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import sys, json, numpy as np
sys.path.insert(0, sys.argv[1])
from kdtree import KDTree
spec = json.loads(sys.argv[2])
rng = np.random.default_rng(spec["seed"])
n, d = spec["n"], spec["d"]
data = rng.uniform(size=(n, d)) if spec["dist"] == "uniform" else None
if data is None:
    c = rng.uniform(size=(64, d)); data = c[rng.integers(0, 64, n)] + 0.01 * rng.standard_normal((n, d))
q = rng.uniform(size=(spec["nq"], d)) * 1.1 - 0.05
out = KDTree(data, leafsize=spec["leafsize"]).query(q, k=spec["k"], p=spec["p"])
np.save(sys.argv[3], np.concatenate([out[0].view(np.int64), out[1]], axis=1))
"""


def _run(spec, mode, tmp_path):
    env = dict(os.environ)
    if mode:
        env["KD_QUERY_MODE"] = mode
    else:
        env.pop("KD_QUERY_MODE", None)
    out = tmp_path / f"out_{mode or 'default'}.npy"
    subprocess.run([sys.executable, "-c", CHILD, str(ROOT / "kdtree-rs_gb300"), json.dumps(spec), str(out)],
                   env=env, check=True)
    arr = np.load(out)
    k = spec["k"]
    return arr[:, :k].view(np.float64), arr[:, k:]


@pytest.mark.parametrize("d", [2, 3, 8])
@pytest.mark.parametrize("p", [1.0, 2.0, float("inf")])
@pytest.mark.parametrize("dist", ["uniform", "gmm"])
def test_packet_and_reference_order_agree(oracle, tmp_path, d, p, dist):
    spec = {"seed": 17 * d + int(p if p != float("inf") else 9), "n": 60_000, "d": d, "nq": 20_000, "k": 16,
            "p": p, "leafsize": 16, "dist": dist}
    packet = _run(spec, None, tmp_path)
    dfs = _run(spec, "dfs", tmp_path)
    assert_bit_exact(packet, dfs)
    rng = np.random.default_rng(spec["seed"])
    n = spec["n"]
    if dist == "uniform":
        data = rng.uniform(size=(n, d))
    else:
        c = rng.uniform(size=(64, d))
        data = c[rng.integers(0, 64, n)] + 0.01 * rng.standard_normal((n, d))
    q = rng.uniform(size=(spec["nq"], d)) * 1.1 - 0.05
    ref = oracle.OracleKDTree(data, leafsize=16).query(q, k=16, p=p, parallel=True)
    assert_bit_exact(packet, ref)


def _path_query(tree, q, k, p, path):
    import ctypes

    import torch

    from kdtree import _core

    L = _core._lib
    P, u64, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double
    L.kd_query_device_path.argtypes = [P, P, u64, u64, dbl, ctypes.c_int, dbl, dbl, P, P, P, ctypes.c_int, P]
    L.kd_query_device_path.restype = ctypes.c_int
    dq = torch.from_numpy(np.ascontiguousarray(q)).cuda()
    od = torch.empty((q.shape[0], k), dtype=torch.float64, device="cuda")
    oi = torch.empty((q.shape[0], k), dtype=torch.int64, device="cuda")
    st = L.kd_query_device_path(tree._h, P(dq.data_ptr()), dq.numel(), k, p, 0, 0.0, 0.0, P(od.data_ptr()),
                                P(oi.data_ptr()), None, path, None)
    assert st == 0, _core._last_error()
    return od.cpu().numpy(), oi.cpu().numpy()


@pytest.mark.parametrize("p", [1.0, 2.0, float("inf")])
@pytest.mark.parametrize("dist", ["uniform", "gmm"])
@pytest.mark.parametrize("k", [1, 4, 8, 16, 32, 50])
def test_packet_width16(oracle, p, dist, k):
    """Width 16 through the packet traversal (Folded L1 / L2 order,
    kernel.rs:343-354) and, for k <= 32, the warp-per-query kernel: bit-exact
    with the oracle."""
    from kdtree import KDTree

    rng = np.random.default_rng(1600 + k)
    data = rng.uniform(size=(30_000, 16)) if dist == "uniform" else gmm(30_000, 16, rng)
    q = data[rng.integers(0, 30_000, 1500)] + 0.02 * rng.standard_normal((1500, 16))
    t = KDTree(data, leafsize=16)
    o = oracle.OracleKDTree(data, leafsize=16).query(q, k=k, p=p, parallel=True)
    assert_bit_exact(_path_query(t, q, k, p, 2), o)  # KD_PATH_PACKET
    assert_bit_exact(_path_query(t, q, k, p, 4), o)  # KD_PATH_WARP


@pytest.mark.parametrize("d", [2, 3, 8])
@pytest.mark.parametrize("p", [1.0, 2.0, float("inf")])
@pytest.mark.parametrize("k", [1, 7, 16, 32, 33, 64])
def test_warp_per_query(oracle, d, p, k):
    """The warp-per-query kernel on uniform and clustered data, queries inside
    and outside the root box, ties on an integer grid."""
    from kdtree import KDTree

    rng = np.random.default_rng(400 + 10 * d + k)
    for data, q in ((rng.uniform(size=(40_000, d)), rng.uniform(size=(2000, d)) * 1.2 - 0.1),
                    (gmm(40_000, d, rng), gmm(2000, d, rng)),
                    (rng.integers(0, 4, size=(5000, d)).astype(float), rng.integers(0, 4, size=(500, d)).astype(float))):
        t = KDTree(data, leafsize=16)
        o = oracle.OracleKDTree(data, leafsize=16).query(q, k=k, p=p, parallel=True)
        assert_bit_exact(_path_query(t, q, k, p, 4), o)
