"""The reference's own test file (tests/test_kdtree.py of FujishigeTemma/kdtree-rs)
run against the GPU engine: every table case and random problems drawn like
its hypothesis strategy, checked against SciPy (the reference's contract:
distances atol 1e-12, indices exact), against the committed golden fixtures,
and bit for bit against the oracle."""
from pathlib import Path

import numpy as np
import pytest

from cases import golden_cases, invalid_cases, random_problem, valid_cases
from helpers import assert_bit_exact, assert_lp_close, assert_reference_contract, scipy_query

pytestmark = pytest.mark.gpu

GOLDEN = np.load(Path(__file__).parent / "golden" / "golden.npz")


def check_query(oracle, data, queries, k, p, max_distance, leafsize, parallel):
    """tests/test_kdtree.py:55-89 of the reference, plus the oracle."""
    from kdtree import KDTree

    actual_tree = KDTree(data, leafsize=leafsize, parallel=parallel)
    actual = actual_tree.query(queries, k=k, p=p, max_distance=max_distance, parallel=parallel)
    expected = scipy_query(data, queries, k, p, max_distance, leafsize)

    assert actual_tree.ndim == data.shape[1]
    assert actual_tree.n_points == data.shape[0]
    assert actual_tree.leafsize == leafsize
    assert len(actual_tree) == data.shape[0]
    np.testing.assert_array_equal(actual_tree.data, data)

    expected_shape = (k,) if np.asarray(queries).ndim == 1 else (np.asarray(queries).shape[0], k)
    assert actual[0].shape == expected_shape
    assert actual[1].shape == expected_shape
    assert actual[0].dtype == np.float64 and actual[1].dtype == np.int64
    assert_reference_contract(actual, expected)

    ot = oracle.OracleKDTree(data, leafsize=leafsize)
    ref = ot.query(queries, k=k, p=p, max_distance=max_distance)
    if p in (1.0, 2.0, np.inf):
        assert_bit_exact(actual, ref)
    else:  # general L^p goes through pow(): within lp_max_ulps ulp (tests/helpers.py)
        assert_lp_close(actual, ref, np.asarray(data).shape[1], p)
    return actual


@pytest.mark.parametrize("name", list(valid_cases()))
def test_valid(oracle, name):
    c = valid_cases()[name]
    got = check_query(oracle, *c)
    np.testing.assert_allclose(got[0], GOLDEN[f"{name}/d"], atol=1e-12)
    np.testing.assert_array_equal(got[1], GOLDEN[f"{name}/i"])


@pytest.mark.parametrize("name", list(invalid_cases()))
def test_invalid(name):
    from kdtree import KDTree

    c = invalid_cases()[name]
    with pytest.raises(ValueError):
        KDTree(c.data, leafsize=c.leafsize).query(c.queries, k=c.k, p=c.p)


@pytest.mark.parametrize("seed", range(100))
def test_compatibility(oracle, seed):
    """tests/test_kdtree.py:92-95 (100 examples), drawn from fixed seeds."""
    check_query(oracle, *random_problem(seed))


def test_plain_small_golden(oracle):
    """N=10,000, d=3, leafsize 32, 1,000 queries, k=8, L2: bit-exact indices."""
    c = golden_cases()["plain-small-n10000-d3-k8"]
    got = check_query(oracle, *c)
    np.testing.assert_array_equal(got[1], GOLDEN["plain-small-n10000-d3-k8/i"])


def test_error_messages():
    """src/error.rs:18-51 texts through the boundary."""
    from kdtree import KDTree

    t = KDTree(np.array([[0.0, 0.0], [1.0, 0.0]]))
    with pytest.raises(ValueError, match=r"^dimension mismatch: expected 2, got 1$"):
        t.query(np.array([0.0]))
    with pytest.raises(ValueError, match=r"^k must be greater than zero$"):
        t.query(np.array([0.0, 0.0]), k=0)
    with pytest.raises(ValueError, match=r"^p must be finite and >= 1, or infinity, got 0.5$"):
        t.query(np.array([0.0, 0.0]), p=0.5)
    with pytest.raises(ValueError, match=r"^p must be finite and >= 1, or infinity, got -inf$"):
        t.query(np.array([0.0, 0.0]), p=-np.inf)
    with pytest.raises(ValueError, match=r"^p must be finite and >= 1, or infinity, got NaN$"):
        t.query(np.array([0.0, 0.0]), p=np.nan)
    with pytest.raises(ValueError, match=r"^eps must be finite and non-negative, got -1$"):
        t.query(np.array([0.0, 0.0]), eps=-1.0)
    with pytest.raises(ValueError, match=r"^max_distance must be finite and non-negative, or infinity, got -0.25$"):
        t.query(np.array([0.0, 0.0]), max_distance=-0.25)
    with pytest.raises(ValueError, match=r"^all coordinates must be finite$"):
        t.query(np.array([np.nan, 0.0]))
    # a non-finite query outranks a bad eps (query.rs:46-50)
    with pytest.raises(ValueError, match=r"^all coordinates must be finite$"):
        t.query(np.array([np.inf, 0.0]), eps=-1.0)
    with pytest.raises(ValueError, match=r"^queries must be a contiguous row-major matrix$"):
        t.query(np.zeros((0, 2)))
    with pytest.raises(ValueError, match=r"^all coordinates must be finite$"):
        KDTree(np.array([[0.0, np.inf]]))
    with pytest.raises(TypeError):
        t.query([0.0, 0.0])
    with pytest.raises(ValueError, match=r"^query must be one- or two-dimensional$"):
        t.query(np.zeros((1, 1, 2)))


def test_repr_and_readonly():
    from kdtree import KDTree

    t = KDTree(np.zeros((5, 3)), leafsize=4)
    assert repr(t) == "KDTree(n_points=5, ndim=3, leafsize=4)"
    with pytest.raises(AttributeError):
        t.ndim = 4
