"""The reference's small-size workload grid (tests/benchmark.py:16-36, 43-108;
benches/grid.rs:257-323), restated: d in {3, 8, 16}, N = 10,000 points,
Q = 1,000 queries, k = 1.

- build cases: "bimodal" (two unit-normal clouds, the second shifted by one in
  every coordinate), "uniform" ([0,1)^d) and "sorted" (row i = (N - i) / N in
  every coordinate, a diagonal line), leafsize 16;
- query cases: uniform and sorted data at leafsize 16, p = 2; uniform data at
  leafsize 8 and 128 with p in {1, 2, inf};
- data seed 123,456,789, query seed 987,654,321, queries uniform in [0,1)^d."""
import numpy as np

SIZES = ((3, 10_000, 1_000), (8, 10_000, 1_000), (16, 10_000, 1_000))
DATA_SEED = 123_456_789
QUERY_SEED = 987_654_321


def make_data(distribution, n_points, dims):
    rng = np.random.default_rng(DATA_SEED)
    if distribution == "bimodal":
        half = n_points // 2
        a = rng.standard_normal((half, dims))
        b = rng.standard_normal((n_points - half, dims)) + 1.0
        return np.concatenate((a, b))
    if distribution == "uniform":
        return rng.uniform(size=(n_points, dims))
    if distribution == "sorted":
        col = np.arange(n_points, 0, -1, dtype=np.float64) / n_points
        return np.repeat(col[:, None], dims, axis=1)
    raise ValueError(distribution)


def make_queries(n_queries, dims):
    return np.random.default_rng(QUERY_SEED).uniform(size=(n_queries, dims))


def build_cases():
    out = []
    for d, n, _ in SIZES:
        for dist in ("bimodal", "uniform", "sorted"):
            out.append((f"build-d{d}-n{n}-{dist}", d, n, dist))
    return out


def query_cases():
    out = []
    for d, n, q in SIZES:
        for dist in ("uniform", "sorted"):
            out.append((f"query-d{d}-n{n}-q{q}-{dist}-leaf16-p2", d, n, q, dist, 16, 2.0))
    for d, n, q in SIZES:
        for p in (1.0, 2.0, float("inf")):
            for leaf in (8, 128):
                pn = "inf" if np.isinf(p) else f"{p:g}"
                out.append((f"query-d{d}-n{n}-q{q}-uniform-leaf{leaf}-p{pn}", d, n, q, "uniform", leaf, p))
    return out
