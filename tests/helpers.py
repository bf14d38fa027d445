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


def lp_max_ulps(d, p):
    """Largest difference, in units in the last place, between an L^p distance
    the GPU returns and the oracle's.  Both follow the reference's operations
    in its order; only pow() differs: CUDA's pow is within 2 ulp, glibc's
    within 0.52, so each term |q_i - p_i|^p differs by at most 2.52 ulp
    (relative).  The sequential sum of d non-negative terms keeps that relative
    bound and adds at most half an ulp of rounding difference per partial sum:
    2.52 + d / 2 ulp.  restore() = pow(sum, 1 / p) divides that by p and adds
    its own 2.52."""
    return int(np.ceil((2.52 + 0.5 * d) / p + 2.52))


def assert_lp_close(actual, expected, d, p):
    """General L^p: indices exact, finite distances within lp_max_ulps(d, p)
    ulp, +inf where the oracle has +inf."""
    a_d, a_i = actual
    e_d, e_i = expected
    np.testing.assert_array_equal(a_i, e_i)
    fin = np.isfinite(e_d)
    assert np.array_equal(np.isfinite(a_d), fin)
    ulps = np.abs(a_d[fin].view(np.int64) - e_d[fin].view(np.int64))
    bound = lp_max_ulps(d, p)
    assert ulps.max(initial=0) <= bound, f"L^p distance off by {ulps.max()} ulp (bound {bound})"


def gmm(n, d, rng, components=64, sigma=0.01):
    """Isotropic Gaussian mixture: centres uniform in [0,1)^d, equal weights."""
    centres = rng.uniform(size=(components, d))
    lab = rng.integers(0, components, size=n)
    return centres[lab] + sigma * rng.standard_normal(size=(n, d))
