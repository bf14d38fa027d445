"""Generate the golden fixtures in this folder.

The reference (FujishigeTemma/kdtree-rs) defines parity as agreement with
`scipy.spatial.KDTree.query(..., distance_upper_bound=max_distance)`: indices
exactly equal, distances within atol 1e-12 (tests/test_kdtree.py:55-89 of the
reference).  The reference itself cannot be built here (no Rust toolchain), so
these fixtures record SciPy's answers on:

- the reference's own table cases (tests/test_kdtree.py:98-164), whose inputs are
  rebuilt by `cases.py` from the same literals and seeds, and
- the small plain workload (N=10,000 uniform [0,1)^3 from seed 0, 1,000 queries
  from seed 1, leafsize 32, k=8, p=2).

Run: python tests/golden/make_golden.py   (writes golden.npz next to this file)
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np
from scipy.spatial import KDTree as SciPyKDTree

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
from cases import golden_cases  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()[:16]


def main():
    out = {}
    for name, c in golden_cases().items():
        data = np.asarray(c.data, dtype=np.float64)
        q = np.asarray(c.queries, dtype=np.float64)
        tree = SciPyKDTree(data, leafsize=c.leafsize)
        d, i = tree.query(q, k=c.k, p=c.p,
                          distance_upper_bound=c.max_distance if c.max_distance is not None else np.inf)
        shape = (c.k,) if q.ndim == 1 else (q.shape[0], c.k)
        out[f"{name}/d"] = np.asarray(d, np.float64).reshape(shape)
        out[f"{name}/i"] = np.asarray(i, np.int64).reshape(shape)
        out[f"{name}/digest"] = np.array(digest(data, q))
    np.savez_compressed(HERE / "golden.npz", **out)
    print(f"wrote {len(out) // 3} cases to {HERE / 'golden.npz'}")


if __name__ == "__main__":
    main()
