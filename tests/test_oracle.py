"""Pinning the CPU oracle (oracle/kd_oracle.c) before it is trusted as the checker.

The oracle is checked against the reference's own test oracle (SciPy) through
the committed golden fixtures of the reference's table cases, on random problems
drawn like the reference's hypothesis strategy, and against a brute-force
(distance, index) sort where SciPy's tie order is not the reference's.
"""
import numpy as np
import pytest

from cases import golden_cases, invalid_cases, random_problem, valid_cases
from helpers import assert_reference_contract, scipy_query

GOLDEN = None


def golden():
    global GOLDEN
    if GOLDEN is None:
        from pathlib import Path

        GOLDEN = np.load(Path(__file__).parent / "golden" / "golden.npz")
    return GOLDEN


def test_golden_inputs_unchanged():
    """The table inputs rebuilt from literals and seeds are the ones the
    fixtures were generated from."""
    from make_golden import digest

    g = golden()
    for name, c in golden_cases().items():
        assert str(g[f"{name}/digest"]) == digest(np.asarray(c.data, np.float64),
                                                   np.asarray(c.queries, np.float64)), name


@pytest.mark.parametrize("name", list(golden_cases()))
def test_oracle_matches_golden(oracle, name):
    c = golden_cases()[name]
    t = oracle.OracleKDTree(c.data, leafsize=c.leafsize, parallel=c.parallel)
    got = t.query(c.queries, k=c.k, p=c.p, max_distance=c.max_distance, parallel=c.parallel)
    g = golden()
    assert_reference_contract(got, (g[f"{name}/d"], g[f"{name}/i"]))
    assert t.ndim == c.data.shape[1] and t.n_points == c.data.shape[0] and len(t) == c.data.shape[0]
    np.testing.assert_array_equal(t.data, c.data)


@pytest.mark.parametrize("name", list(invalid_cases()))
def test_oracle_invalid(oracle, name):
    c = invalid_cases()[name]
    with pytest.raises(ValueError):
        oracle.OracleKDTree(c.data, leafsize=c.leafsize).query(c.queries, k=c.k, p=c.p)


@pytest.mark.parametrize("seed", range(60))
def test_oracle_random_problems(oracle, seed):
    c = random_problem(seed)
    t = oracle.OracleKDTree(c.data, leafsize=c.leafsize, parallel=c.parallel)
    got = t.query(c.queries, k=c.k, p=c.p, max_distance=c.max_distance, parallel=c.parallel)
    assert_reference_contract(got, scipy_query(c.data, c.queries, c.k, c.p, c.max_distance, c.leafsize))


def test_oracle_hypothesis(oracle):
    """The reference's property test (tests/test_kdtree.py:92-95), fewer examples."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=40, deadline=None)
    @hyp.given(seed=st.integers(0, 2**32 - 1))
    def run(seed):
        c = random_problem(seed)
        t = oracle.OracleKDTree(c.data, leafsize=c.leafsize, parallel=c.parallel)
        got = t.query(c.queries, k=c.k, p=c.p, max_distance=c.max_distance, parallel=c.parallel)
        assert_reference_contract(got, scipy_query(c.data, c.queries, c.k, c.p, c.max_distance, c.leafsize))

    run()


def _brute(data, q, k, p):
    diff = np.abs(q[:, None, :] - data[None, :, :])
    if np.isinf(p):
        d = diff.max(-1)
    elif p == 1:
        d = diff.sum(-1)
    else:
        d = np.sqrt((diff**2).sum(-1))
    idx = np.argsort(d, axis=1, kind="stable")[:, :k]  # stable: ties in index order
    return np.take_along_axis(d, idx, 1), idx


@pytest.mark.parametrize("p", [1.0, 2.0, np.inf])
@pytest.mark.parametrize("leafsize", [1, 4, 16])
def test_oracle_tie_order(oracle, p, leafsize):
    """Integer-grid data: exact distance ties everywhere; the (dist, idx) order
    of query.rs:384-386 decides (SciPy does not order ties by index)."""
    rng = np.random.default_rng(5)
    data = rng.integers(0, 4, size=(3000, 3)).astype(float)
    q = rng.integers(0, 4, size=(50, 3)).astype(float)
    got = oracle.OracleKDTree(data, leafsize=leafsize).query(q, k=7, p=p)
    exp = _brute(data, q, 7, p)
    np.testing.assert_array_equal(got[1], exp[1])
    np.testing.assert_allclose(got[0], exp[0], atol=1e-12)


def test_oracle_parallel_build_matches_serial(oracle):
    """build.rs:345-359: bit-identical data, indices, nodes and boxes."""
    data = ((np.arange(2000 * 5) * 2_654_435_761) % 10_007).astype(np.float64).reshape(2000, 5)
    a = oracle.OracleKDTree(data, leafsize=8).export()
    b = oracle.OracleKDTree(data, leafsize=8, parallel=True).export()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_oracle_rejects_empty(oracle):
    """build.rs:320-323."""
    with pytest.raises(ValueError):
        oracle.OracleKDTree(np.zeros((0, 2)))


def _count_nodes_naive(n, ls):
    return 1 if n <= ls else 1 + _count_nodes_naive(n // 2, ls) + _count_nodes_naive(n - n // 2, ls)


@pytest.mark.parametrize("ls", [1, 2, 3, 16, 32])
def test_count_nodes(oracle, ls):
    for n in list(range(1, 300)) + [1000, 4097, 10_000]:
        assert oracle.count_nodes(n, ls) == _count_nodes_naive(n, ls)


def test_valid_cases_cover_every_strategy():
    """The row-width cases span Packed (d<=8), Folded (9..16) and Streamed (17)."""
    dims = {c.data.shape[1] for n, c in valid_cases().items() if n.startswith("row-width")}
    assert dims == set(range(1, 18))


def _adversarial():
    from pathlib import Path

    f = np.load(Path(__file__).parent / "golden" / "adversarial.npz")
    out = []
    for i in range(int(f["n_cases"])):
        leaf, k, p, md = f[f"c{i}_params"]
        out.append((f[f"c{i}_data"], f[f"c{i}_q"], int(leaf), int(k), float(p),
                    None if np.isnan(md) else float(md), f[f"c{i}_ref_d"], f[f"c{i}_ref_i"]))
    return out


@pytest.mark.parametrize("case", range(19))
def test_oracle_adversarial_gate_rounding(oracle, case):
    """tests/golden/adversarial.npz (make_adversarial.py): the oracle still
    returns the recorded answer, and the brute-force top-k over every point
    differs on at least one query -- the reference's descent prunes a point
    there because one of its FP64 gates rounds above that point's distance."""
    data, q, leaf, k, p, md, ref_d, ref_i = _adversarial()[case]
    t = oracle.OracleKDTree(data, leafsize=leaf)
    got = t.query(q, k=k, p=p, max_distance=md)
    np.testing.assert_array_equal(got[1], ref_i)
    assert np.array_equal(got[0], ref_d)
    bru = t.query_brute(q, k=k, p=p, max_distance=md)
    assert not (np.array_equal(bru[1], ref_i) and np.array_equal(bru[0], ref_d))
    # and the difference is a tie or near-tie at the k-th place or the cutoff:
    # the brute force's extra point sits within 2^-40 (relative) of the
    # distance the two answers disagree at, of the one before it, or of the cutoff
    rows = np.nonzero((bru[1] != ref_i).any(1))[0]
    for r in rows:
        j = int(np.argmax(bru[1][r] != ref_i[r]))
        b = bru[0][r][j]
        near = [x for x in (ref_d[r][j], md if md is not None else np.inf) if np.isfinite(x)]
        if j > 0:
            near.append(ref_d[r][j - 1])
        assert any(abs(b - x) <= 2.0 ** -40 * max(abs(x), 1e-300) for x in near)
