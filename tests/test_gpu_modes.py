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
