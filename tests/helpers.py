"""Shared assertions for the parity tests."""
from __future__ import annotations

import numpy as np
from scipy.spatial import KDTree as SciPyKDTree


def scipy_query(data, queries, k, p, max_distance, leafsize):
    """The reference's own test oracle (tests/test_kdtree.py:67-74 of the reference)."""
    data = np.asarray(data, np.float64)
    q = np.asarray(queries, np.float64)
    t = SciPyKDTree(data, leafsize=leafsize)
    d, i = t.query(q, k=k, p=p, distance_upper_bound=max_distance if max_distance is not None else np.inf)
    shape = (k,) if q.ndim == 1 else (q.shape[0], k)
    return np.asarray(d).reshape(shape), np.asarray(i).reshape(shape)


def assert_reference_contract(actual, expected):
    """tests/test_kdtree.py:86-89 of the reference: distances atol 1e-12, indices exact."""
    np.testing.assert_allclose(actual[0], expected[0], atol=1e-12)
    np.testing.assert_array_equal(actual[1], expected[1])


def assert_bit_exact(actual, expected):
    """Distances bit-identical (as float64 values; -0 == +0) and indices equal."""
    a_d, a_i = actual
    e_d, e_i = expected
    assert a_d.shape == e_d.shape and a_i.shape == e_i.shape
    bad = ~((a_d == e_d) | (np.isnan(a_d) & np.isnan(e_d)))
    if bad.any():
        w = np.argwhere(bad)[:5]
        raise AssertionError(f"{bad.sum()} distances differ, first at {w.tolist()}: "
                             f"{a_d[bad][:5]} vs {e_d[bad][:5]}")
    np.testing.assert_array_equal(a_i, e_i)


def gmm(n, d, rng, components=64, sigma=0.01):
    """Isotropic Gaussian mixture: centres uniform in [0,1)^d, equal weights."""
    centres = rng.uniform(size=(components, d))
    lab = rng.integers(0, components, size=n)
    return centres[lab] + sigma * rng.standard_normal(size=(n, d))
