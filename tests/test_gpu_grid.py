"""The reference's small-size workload grid through the engine: every build
case's layout and every query case's results bit-exact against the oracle."""
import numpy as np
import pytest

from grid_workloads import build_cases, make_data, make_queries, query_cases
from helpers import assert_bit_exact

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,d,n,dist", build_cases(), ids=[c[0] for c in build_cases()])
def test_grid_build(oracle, name, d, n, dist):
    from kdtree import KDTree

    data = make_data(dist, n, d)
    g = KDTree(data, leafsize=16)._export()
    o = oracle.OracleKDTree(data, leafsize=16).export()
    for a, b in zip(g, o):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name,d,n,q,dist,leaf,p", query_cases(), ids=[c[0] for c in query_cases()])
def test_grid_query(oracle, name, d, n, q, dist, leaf, p):
    from kdtree import KDTree

    data = make_data(dist, n, d)
    qs = make_queries(q, d)
    for parallel in (False, True):
        g = KDTree(data, leafsize=leaf).query(qs, k=1, p=p, parallel=parallel)
        o = oracle.OracleKDTree(data, leafsize=leaf).query(qs, k=1, p=p, parallel=True)
        assert_bit_exact(g, o)
