"""Generate tests/golden/adversarial.npz: inputs on which the reference's
descent prunes a point that an exact top-k keeps.

The reference's descent (src/query.rs:223-341) skips a subtree when one of its
FP64 gates -- the root seed (query.rs:169-194), the split-plane bound
`replace_axis` (metric.rs:93-98) or the box distance (kernel.rs:565-616) --
exceeds the current bound.  Each gate is a rounded lower bound of the exact
distance to the subtree, and it can round a few ulps ABOVE the distance of a
point inside, as the leaf scan computes it in its own summation order
(kernel.rs:163-218, 343-562).  When that point ties the k-th distance or the
cutoff, the reference leaves it out.  The search below finds such inputs:
small point sets on a coarse lattice of awkward decimals (many equal
distances), queries on and off the lattice, and cutoffs set to exact
distances.  A case is kept when the oracle (the restatement of the reference's
descent) and `query_brute` (every point, same per-point arithmetic) disagree.

The fixture holds, per case, the points, a 32-query batch, leafsize, k, p,
max_distance (NaN for None) and the oracle's answer for every query of the
batch.  It is the reference's answer for these inputs: tests check the oracle
still gives it, that the brute force differs (so the case stays adversarial),
and that the GPU engine returns it on every query path.

Run from the repository root: python tests/golden/make_adversarial.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import kdtree_oracle as ko  # noqa: E402

OUT = Path(__file__).resolve().parent / "adversarial.npz"
# (d, p) classes and how many divergent cases to keep of each
CLASSES = {(2, 1.0): 2, (2, 2.0): 2, (3, 1.0): 2, (3, 2.0): 3, (8, 1.0): 2, (8, 2.0): 2,
           (20, 2.0): 2, (64, 2.0): 2, (64, 1.0): 1}
NQ = 32


def lattice_case(rng, d):
    n = int(rng.integers(8, 300))
    leaf = int(rng.choice([1, 2, 4, 8, 16]))
    vals = rng.uniform(0, 1, int(rng.integers(3, 12))) * rng.choice([1.0, 0.1, 10.0, 1e-3])
    data = rng.choice(vals, (n, d))
    if rng.random() < 0.5:
        q = rng.choice(vals, (NQ, d)) + rng.choice([0, 0, 1e-9, -1e-9], (NQ, d))
    else:
        q = rng.uniform(vals.min() - 0.5, vals.max() + 0.5, (NQ, d))
    return data, q, leaf


def root_seed_case():
    """The root gate alone (d = 8, L1): the query lies below the root box in
    every dimension, so the descent starts from the seed, a sequential sum of
    the eight axis offsets (query.rs:177-187); the box's corner point p* has the
    same offsets, summed in the Packed d8 pairwise order (kernel.rs:540-562).
    With max_distance = dist(p*) and the seed one ulp above it, the reference
    never enters the root."""
    rng = np.random.default_rng(0)
    for _ in range(100_000):
        q = rng.uniform(0, 0.3, 8)
        ps = rng.uniform(0.3, 0.6, 8)
        off = [float(ps[i] - q[i]) for i in range(8)]
        seed = 0.0
        for v in off:
            seed += v
        a = [abs(float(q[i] - ps[i])) for i in range(8)]
        dist = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]))
        if seed > dist:
            data = np.vstack([ps] + [ps + rng.uniform(0.5, 1.0, 8) for _ in range(7)])
            qs = np.vstack([q] + [rng.uniform(0, 1.5, 8) for _ in range(NQ - 1)])
            return data, qs, 8, 1, 1.0, dist
    raise RuntimeError("no root-seed case found")


def main():
    rng = np.random.default_rng(20261204)
    need = dict(CLASSES)
    cases = []
    data, q, leaf, k, p, md = root_seed_case()
    t = ko.OracleKDTree(data, leafsize=leaf)
    cases.append((data, q, leaf, k, p, md) + t.query(q, k=k, p=p, max_distance=md))
    tries = 0
    while any(v > 0 for v in need.values()):
        tries += 1
        if tries > 200_000:
            raise RuntimeError(f"search gave up; still missing {need}")
        d, p = list(need)[int(rng.integers(len(need)))]
        if need[(d, p)] == 0:
            continue
        data, q, leaf = lattice_case(rng, d)
        k = int(rng.choice([1, 2, 3, 5, 8]))
        t = ko.OracleKDTree(data, leafsize=leaf)
        n = data.shape[0]
        bd, _ = t.query_brute(q, k=min(n, k + 2), p=p)
        md = float(bd[0][int(rng.integers(0, min(n, k + 2)))]) if rng.random() < 0.6 else None
        ref = t.query(q, k=k, p=p, max_distance=md)
        bru = t.query_brute(q, k=k, p=p, max_distance=md)
        if np.array_equal(ref[1], bru[1]) and np.array_equal(ref[0], bru[0]):
            continue
        cases.append((data, q, leaf, k, p, np.nan if md is None else md) + ref)
        need[(d, p)] -= 1
    arrays = {}
    for i, (data, q, leaf, k, p, md, ref_d, ref_i) in enumerate(cases):
        arrays[f"c{i}_data"] = data
        arrays[f"c{i}_q"] = q
        arrays[f"c{i}_params"] = np.array([leaf, k, p, md], np.float64)
        arrays[f"c{i}_ref_d"] = ref_d
        arrays[f"c{i}_ref_i"] = ref_i
    arrays["n_cases"] = np.array(len(cases))
    np.savez_compressed(OUT, **arrays)
    print(f"{len(cases)} cases -> {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
