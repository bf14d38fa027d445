"""The reference's table cases (tests/test_kdtree.py:98-169 of
FujishigeTemma/kdtree-rs), rebuilt from the same literals and seeds, plus the
small plain workload.  Shared by the golden-fixture generator and the tests."""
from __future__ import annotations

from typing import NamedTuple

import numpy as np


class Case(NamedTuple):
    data: np.ndarray
    queries: np.ndarray
    k: int = 1
    p: float = 2.0
    max_distance: float | None = None
    leafsize: int = 32
    parallel: bool = False


def valid_cases() -> dict[str, Case]:
    """tests/test_kdtree.py:98-164 of the reference."""
    return {
        "single-query": Case(np.array([[0.0, 0.0], [1.0, 0.0], [4.0, 0.0]]), np.array([0.2, 0.0]), k=2),
        "batch-query": Case(np.array([[0.0, 0.0], [1.0, 0.0], [4.0, 0.0]]),
                            np.array([[0.2, 0.0], [3.8, 0.0]]), k=2),
        "max-distance-padding": Case(np.array([[0.0, 0.0], [5.0, 0.0], [10.0, 0.0]]), np.array([0.0, 0.0]),
                                     k=3, max_distance=1.0),
        "infinite-norm": Case(np.array([[0.0, 0.0], [2.0, 1.0], [1.0, 2.0]]), np.array([[0.1, 0.8]]), k=3,
                              p=np.inf, leafsize=1),
        "single-query-k1": Case(np.array([[0.0, 0.0], [1.0, 0.0], [4.0, 0.0]]), np.array([0.2, 0.0])),
        "batch-query-k1": Case(np.array([[0.0, 0.0], [1.0, 0.0], [4.0, 0.0]]), np.array([[0.2, 0.0], [3.8, 0.0]])),
        "k-greater-than-points": Case(np.array([[0.0], [2.0]]), np.array([[0.5]]), k=4),
        "promoted-dtype": Case(np.array([[0, 0], [1, 0], [4, 0]], dtype=np.int64),
                               np.array([[0.2, 0.0]], dtype=np.float32), k=2),
        "non-contiguous": Case(np.asfortranarray([[0.0, 0.0], [1.0, 0.0], [4.0, 0.0]]),
                               np.array([[0.2, 9.0, 0.0], [3.8, 9.0, 0.0]])[:, ::2], k=2),
        "large-parallel-batch": Case(np.random.default_rng(0).normal(size=(2_000, 8)),
                                     np.random.default_rng(1).normal(size=(256, 8)), k=4, parallel=True),
        **{
            f"row-width-{dims:02d}-p{'inf' if np.isinf(p) else int(p)}": Case(
                np.random.default_rng(dims).normal(size=(512, dims)),
                np.random.default_rng(1_000 + dims).normal(size=(64, dims)),
                k=3, p=p, leafsize=6)
            for dims in range(1, 18)
            for p in (1.0, 2.0, np.inf)
        },
    }


def invalid_cases() -> dict[str, Case]:
    """tests/test_kdtree.py:166-169 of the reference."""
    return {
        "query-wrong-dimensions": Case(np.array([[0.0, 0.0], [1.0, 0.0]]), np.array([0.0])),
        "zero-k": Case(np.array([[0.0, 0.0], [1.0, 0.0]]), np.array([0.0, 0.0]), k=0),
    }


def plain_small() -> Case:
    """N=10,000 uniform [0,1)^3 (seed 0), 1,000 queries (seed 1), leafsize 32, k=8, L2."""
    return Case(np.random.default_rng(0).uniform(size=(10_000, 3)),
                np.random.default_rng(1).uniform(size=(1_000, 3)), k=8, p=2.0, leafsize=32)


def golden_cases() -> dict[str, Case]:
    cases = dict(valid_cases())
    cases["plain-small-n10000-d3-k8"] = plain_small()
    return cases


def random_problem(seed: int):
    """One problem drawn like the reference's hypothesis strategy
    (tests/test_kdtree.py:33-52): dims 1-20, N 1-10,000, 1-32 normal queries
    (sometimes a single 1-D query), k 1-16, p in {1, 2, 3, inf}, max_distance
    None or [0, 4], leafsize in {1, 8, 16, 32, 64}, parallel either."""
    r = np.random.default_rng(seed)
    dims = int(r.integers(1, 21))
    n_points = int(r.integers(1, 10_001))
    n_queries = int(r.integers(1, 33))
    rng = np.random.default_rng(int(r.integers(0, 2**32)))
    queries = rng.normal(size=(n_queries, dims))
    if r.integers(0, 2):
        queries = queries[0]
    return Case(
        data=rng.normal(size=(n_points, dims)),
        queries=queries,
        k=int(r.integers(1, 17)),
        p=float([1.0, 2.0, 3.0, np.inf][int(r.integers(0, 4))]),
        max_distance=None if r.integers(0, 2) else float(r.uniform(0.0, 4.0)),
        leafsize=int([1, 8, 16, 32, 64][int(r.integers(0, 5))]),
        parallel=bool(r.integers(0, 2)),
    )
