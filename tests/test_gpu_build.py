"""GPU build layout against the oracle, array by array and bit for bit:
tree-ordered rows, original indices, node records (including order_by_box),
split values and per-node boxes (src/build.rs, src/tree.rs, src/layout.rs).

The cases cover the one-CTA subtree path (segments <= 8192 rows, split by the
whole CTA above 512 rows and by one warp below), the multi-CTA path of the top
levels, a leaves-only last level below them (large leafsize), the pivot-equal fix-up of partition_rows in
both (duplicated coordinates), a root that is a leaf, leafsize 1, widths 1 to
64, data on a line that sets order_by_box, and the parallel flag."""
import zlib

import numpy as np
import pytest

from helpers import gmm

pytestmark = pytest.mark.gpu


def _compare(oracle, data, leafsize, parallel=False):
    from kdtree import KDTree

    g = KDTree(data, leafsize=leafsize, parallel=parallel)._export()
    o = oracle.OracleKDTree(data, leafsize=leafsize).export()
    names = ("data", "indices", "node words", "split values", "boxes")
    for name, a, b in zip(names, g, o):
        assert a.shape == b.shape, name
        if a.dtype.kind == "f":
            same = (a == b)
            assert same.all(), f"{name}: {np.count_nonzero(~same)} of {a.size} differ"
        else:
            np.testing.assert_array_equal(a, b, err_msg=name)
    return g


CASES = {
    "tiny-root-leaf": (lambda r: r.normal(size=(5, 3)), 32),
    "leafsize-1": (lambda r: r.normal(size=(300, 2)), 1),
    "d1": (lambda r: r.normal(size=(4000, 1)), 8),
    "d3-small-path": (lambda r: r.uniform(size=(5000, 3)), 16),
    "d3-large-path": (lambda r: r.uniform(size=(200_000, 3)), 16),
    "d5-odd-leafsize": (lambda r: r.normal(size=(30_000, 5)), 7),
    "d8": (lambda r: r.normal(size=(50_000, 8)), 16),
    "d17": (lambda r: r.normal(size=(20_000, 17)), 32),
    "d64": (lambda r: r.normal(size=(20_000, 64)) * np.exp(r.uniform(np.log(0.1), np.log(10), 64)), 16),
    "gmm": (lambda r: gmm(100_000, 3, r), 16),
    "diagonal-order-by-box": (lambda r: (lambda t: np.c_[t, t + 1e-3 * r.normal(size=t.size),
                                                         t + 1e-3 * r.normal(size=t.size)])(r.uniform(size=60_000)), 16),
    "dups-small": (lambda r: r.integers(0, 4, size=(6000, 3)).astype(float), 4),
    "dups-large": (lambda r: r.integers(0, 3, size=(60_000, 3)).astype(float), 16),
    "dups-one-coordinate": (lambda r: np.c_[np.zeros(40_000), r.normal(size=40_000)], 16),
    "all-equal": (lambda r: np.ones((20_000, 2)), 8),
    "grid-ties": (lambda r: np.stack(np.meshgrid(np.arange(40.0), np.arange(40.0)), -1).reshape(-1, 2), 3),
    "large-leafsize": (lambda r: r.normal(size=(50_000, 2)), 10_000),
    "big-range": (lambda r: r.normal(size=(10_000, 3)) * 1e300, 16),
    "root-leaf-above-8192": (lambda r: r.normal(size=(9000, 2)), 10_000),
    "n-8192": (lambda r: r.uniform(size=(8192, 3)), 16),
    "n-8193": (lambda r: r.uniform(size=(8193, 3)), 16),
    "signed-zeros": (lambda r: r.choice([-0.0, 0.0, 1.0, -1.0], size=(20_000, 2)), 8),
}


@pytest.mark.parametrize("name", list(CASES))
def test_build_layout_matches_oracle(oracle, name):
    make, leafsize = CASES[name]
    data = make(np.random.default_rng(zlib.crc32(name.encode())))
    g = _compare(oracle, data, leafsize)
    if name == "diagonal-order-by-box":
        assert (g[2][:, 3] >> 31).any(), "clustered data should set order_by_box somewhere"


def test_build_parallel_flag_is_identical(oracle):
    data = ((np.arange(2000 * 5) * 2_654_435_761) % 10_007).astype(np.float64).reshape(2000, 5)
    _compare(oracle, data, 8, parallel=True)


def test_original_data_roundtrip():
    from kdtree import KDTree

    data = np.random.default_rng(3).normal(size=(123_457, 4))
    t = KDTree(data, leafsize=16)
    np.testing.assert_array_equal(t.data, data)


def test_build_full_size_properties():
    """N=1M, d=3, leafsize 16: every leaf holds 15 or 16 rows, the rows are a
    permutation of the input, and every row lies in its leaf's box."""
    from kdtree import KDTree

    data = np.random.default_rng(2).uniform(size=(1_000_000, 3))
    t = KDTree(data, leafsize=16)
    rows, idx, words, split, boxes = t._export()
    assert words.shape[0] == 131_071
    np.testing.assert_array_equal(np.sort(idx), np.arange(1_000_000, dtype=np.uint32))
    np.testing.assert_array_equal(rows, data[idx])
    leaves = words[:, 0] == 1
    lens = words[leaves, 2] - words[leaves, 1]
    assert set(np.unique(lens)) <= {15, 16}
    starts = words[leaves, 1]
    owner = np.repeat(np.nonzero(leaves)[0], lens)
    pos = np.concatenate([np.arange(s, s + n) for s, n in zip(starts, lens)])
    assert np.all(rows[pos] >= boxes[owner, 0]) and np.all(rows[pos] <= boxes[owner, 1])
