"""ctypes wrapper around the CPU oracle (oracle/kd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by `__graft_entry__.smoke()` and
by bench.py's CPU-baseline leg, never by the `kdtree` package.  It mirrors the
reference's Python surface (`src/lib.rs:100-183`: `KDTree(data, *, leafsize,
parallel)`, `.query(x, *, k, p, max_distance, eps, parallel)`) so the parity
tests read like the reference's own `tests/test_kdtree.py`.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libkdoracle.so"
_lib = None

# Status codes shared with include/kdtree_gb300.h (KD_*).
STATUS_NAMES = {
    0: "OK",
    1: "EmptyData",
    2: "InvalidLeafsize",
    3: "InvalidK",
    4: "InvalidMetric",
    5: "InvalidEps",
    6: "InvalidMaxDistance",
    7: "NonFiniteData",
    8: "TooManyPoints",
    9: "TooManyNodes",
    10: "InvalidShape",
    101: "OutOfMemory",
}


class OracleError(ValueError):
    def __init__(self, status: int):
        super().__init__(STATUS_NAMES.get(status, f"status {status}"))
        self.status = status


def build_oracle() -> Path:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists() or _LIB_PATH.stat().st_mtime < (_HERE / "kd_oracle.c").stat().st_mtime:
            build_oracle()
        L = ctypes.CDLL(str(_LIB_PATH))
        P = ctypes.c_void_p
        u64 = ctypes.c_uint64
        L.ork_build.argtypes = [P, u64, u64, u64, ctypes.c_int, ctypes.POINTER(P)]
        L.ork_build.restype = ctypes.c_int
        L.ork_query.argtypes = [P, P, u64, u64, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, P, P, P]
        L.ork_query.restype = ctypes.c_int
        L.ork_query_brute.argtypes = [P, P, u64, u64, ctypes.c_double, ctypes.c_int, ctypes.c_double, P, P]
        L.ork_query_brute.restype = ctypes.c_int
        L.ork_free.argtypes = [P]
        L.ork_info.argtypes = [P, P, P, P, P]
        L.ork_export.argtypes = [P, P, P, P, P, P]
        L.ork_original_data.argtypes = [P, P]
        L.ork_count_nodes.argtypes = [u64, u64]
        L.ork_count_nodes.restype = u64
        L.ork_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().ork_max_threads())


def count_nodes(n: int, leafsize: int) -> int:
    return int(lib().ork_count_nodes(n, leafsize))


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _as_points(obj, allow_single: bool, what: str):
    """src/lib.rs:25-72: any ndarray, promoted to float64, copied row-major."""
    if not isinstance(obj, np.ndarray):
        raise TypeError(f"expected a numpy.ndarray, got {type(obj).__name__}")
    a = np.ascontiguousarray(obj.astype(np.float64, copy=False))
    if a.ndim == 1 and allow_single:
        return a.reshape(1, -1), True
    if a.ndim == 2:
        return a, False
    raise ValueError(what)


class OracleKDTree:
    """The oracle behind the reference's `KDTree` surface."""

    def __init__(self, data, *, leafsize: int = 32, parallel: bool = False):
        pts, _ = _as_points(data, False, "data must be a two-dimensional array")
        self._ptr = ctypes.c_void_p()
        st = lib().ork_build(_ptr(pts), pts.size, pts.shape[1], int(leafsize), int(bool(parallel)),
                             ctypes.byref(self._ptr))
        if st:
            raise OracleError(st)
        n, d, ls, nn = (np.zeros(1, np.uint64) for _ in range(4))
        lib().ork_info(self._ptr, _ptr(n), _ptr(d), _ptr(ls), _ptr(nn))
        self.n_points, self.ndim, self.leafsize, self.n_nodes = int(n[0]), int(d[0]), int(ls[0]), int(nn[0])
        self.last_counts = None

    def __del__(self):
        p = getattr(self, "_ptr", None)
        if p and _lib is not None:
            _lib.ork_free(p)
            self._ptr = None

    def __len__(self):
        return self.n_points

    @property
    def data(self) -> np.ndarray:
        out = np.empty((self.n_points, self.ndim), np.float64)
        lib().ork_original_data(self._ptr, _ptr(out))
        return out

    def export(self):
        """(data in tree order, indices, node words [n_nodes, 4], split values, boxes)."""
        data = np.empty((self.n_points, self.ndim), np.float64)
        idx = np.empty(self.n_points, np.uint32)
        words = np.empty((self.n_nodes, 4), np.uint32)
        split = np.empty(self.n_nodes, np.float64)
        boxes = np.empty((self.n_nodes, 2, self.ndim), np.float64)
        lib().ork_export(self._ptr, _ptr(data), _ptr(idx), _ptr(words), _ptr(split), _ptr(boxes))
        return data, idx, words, split, boxes

    def query(self, x, *, k: int = 1, p: float = 2.0, max_distance=None, eps: float = 0.0,
              parallel: bool = False, threads: int | None = None):
        q, single = _as_points(x, True, "query must be one- or two-dimensional")
        if q.shape[1] != self.ndim:
            raise ValueError(f"dimension mismatch: expected {self.ndim}, got {q.shape[1]}")
        k = int(k)
        nq = q.shape[0]
        out_d = np.empty((max(nq, 1), max(k, 1)), np.float64)
        out_i = np.empty((max(nq, 1), max(k, 1)), np.int64)
        counts = np.zeros(3, np.uint64)
        if threads is None:
            threads = max_threads() if parallel else 1
        st = lib().ork_query(self._ptr, _ptr(q), q.size, k, float(p), int(max_distance is not None),
                             float(max_distance) if max_distance is not None else 0.0, float(eps),
                             int(threads), _ptr(out_d), _ptr(out_i), _ptr(counts))
        if st:
            raise OracleError(st)
        self.last_counts = tuple(int(c) for c in counts)
        if single:
            return out_d[0], out_i[0]
        return out_d, out_i

    def query_brute(self, x, *, k: int = 1, p: float = 2.0, max_distance=None):
        """The exact top-k over every point (each distance as the reference's
        leaf scan computes it), without the descent: the reference's answer
        unless one of its FP64 gates rounds above a point it would keep."""
        q, single = _as_points(x, True, "query must be one- or two-dimensional")
        k = int(k)
        nq = q.shape[0]
        out_d = np.empty((nq, k), np.float64)
        out_i = np.empty((nq, k), np.int64)
        st = lib().ork_query_brute(self._ptr, _ptr(q), q.size, k, float(p), int(max_distance is not None),
                                   float(max_distance) if max_distance is not None else 0.0, _ptr(out_d),
                                   _ptr(out_i))
        if st:
            raise OracleError(st)
        if single:
            return out_d[0], out_i[0]
        return out_d, out_i


if os.environ.get("KD_ORACLE_BUILD_ON_IMPORT"):
    build_oracle()
