"""`KDTree` over the GB300 engine's C ABI (include/kdtree_gb300.h).

Restates the reference's pyo3 boundary (src/lib.rs:1-190) on top of
libkdtree_gb300.so through ctypes:

- inputs: any numpy.ndarray, promoted with `astype("float64")` and copied
  row-major (lib.rs:25-45); anything else raises TypeError;
- `data` must be 2-D, a query 1-D (single point) or 2-D (lib.rs:54-72), and a
  query of the wrong width raises ValueError("dimension mismatch: ...")
  (lib.rs:74-84);
- reference errors (src/error.rs) raise ValueError with the reference's text;
- results are fresh float64 / int64 arrays of shape (n, k), or (k,) for a 1-D
  query (lib.rs:161-182);
- ctypes releases the GIL for the duration of every native call, as
  `py.detach` does in the reference (lib.rs:117, 176).

There is no CPU fallback: a missing library raises ImportError, a machine
without a CUDA device raises RuntimeError on the first build.
"""
from __future__ import annotations

import ctypes
import operator
import weakref
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent.parent / "_build" / "libkdtree_gb300.so"

# Status codes (include/kdtree_gb300.h).  1..11 are the reference's KDTreeError.
KD_OK = 0
_VALUE_ERRORS = set(range(1, 12))
KD_ERR_OUT_OF_MEMORY = 101


def _load():
    if not _LIB_PATH.exists():
        raise ImportError(
            f"{_LIB_PATH} is missing: build the CUDA engine first "
            "(python kdtree-rs_gb300/build_lib.py); there is no CPU fallback"
        )
    L = ctypes.CDLL(str(_LIB_PATH))
    P = ctypes.c_void_p
    u64 = ctypes.c_uint64
    d = ctypes.c_double
    L.kd_build.argtypes = [P, u64, u64, u64, ctypes.c_int, ctypes.POINTER(P)]
    L.kd_build.restype = ctypes.c_int
    L.kd_build_device.argtypes = [P, u64, u64, u64, P, ctypes.POINTER(P)]
    L.kd_build_device.restype = ctypes.c_int
    L.kd_free.argtypes = [P]
    L.kd_free.restype = None
    L.kd_query.argtypes = [P, P, u64, u64, d, ctypes.c_int, d, d, ctypes.c_int, P, P]
    L.kd_query.restype = ctypes.c_int
    L.kd_query_device.argtypes = [P, P, u64, u64, d, ctypes.c_int, d, d, P, P, P]
    L.kd_query_device.restype = ctypes.c_int
    L.kd_query_async.argtypes = [P, P, u64, u64, d, ctypes.c_int, d, d, P, P, P, P]
    L.kd_query_async.restype = ctypes.c_int
    for name in ("kd_ndim", "kd_n_points", "kd_leafsize", "kd_n_nodes"):
        getattr(L, name).argtypes = [P]
        getattr(L, name).restype = u64
    L.kd_count_nodes.argtypes = [u64, u64]
    L.kd_count_nodes.restype = u64
    L.kd_original_data.argtypes = [P, P]
    L.kd_original_data.restype = ctypes.c_int
    L.kd_export.argtypes = [P, P, P, P, P, P]
    L.kd_export.restype = ctypes.c_int
    L.kd_batch_create.argtypes = [P, u64, d, ctypes.c_int, d, d, ctypes.POINTER(P)]
    L.kd_batch_create.restype = ctypes.c_int
    L.kd_batch_run_mode.argtypes = [P, P, ctypes.c_int]
    L.kd_batch_run_mode.restype = ctypes.c_int
    L.kd_batch_free.argtypes = [P]
    L.kd_batch_free.restype = None
    L.kd_batch_choice.argtypes = [P, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_uint)]
    L.kd_batch_choice.restype = ctypes.c_int
    L.kd_server_create.argtypes = [P, u64, d, ctypes.c_int, d, d, u64, ctypes.POINTER(P)]
    L.kd_server_create.restype = ctypes.c_int
    L.kd_server_submit.argtypes = [P, u64, P, u64, u64, P, P, ctypes.POINTER(u64)]
    L.kd_server_submit.restype = ctypes.c_int
    L.kd_server_wait.argtypes = [P, u64, ctypes.POINTER(d)]
    L.kd_server_wait.restype = ctypes.c_int
    L.kd_server_free.argtypes = [P]
    L.kd_server_free.restype = None
    L.kd_host_alloc.argtypes = [u64, ctypes.POINTER(P)]
    L.kd_host_alloc.restype = ctypes.c_int
    L.kd_host_free.argtypes = [P]
    L.kd_host_free.restype = None
    L.kd_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.kd_last_error.restype = ctypes.c_size_t
    return L


_lib = _load()


def library_path() -> Path:
    return _LIB_PATH


def _last_error() -> str:
    n = _lib.kd_last_error(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    _lib.kd_last_error(buf, n + 1)
    return buf.value.decode("utf-8", "replace")


def _raise(status: int):
    msg = _last_error()
    if status in _VALUE_ERRORS:
        raise ValueError(msg)
    if status == KD_ERR_OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise RuntimeError(f"kdtree engine error {status}: {msg}")


def _usize(v, name: str) -> int:
    """pyo3's `usize` extraction: an integer (TypeError otherwise) >= 0
    (OverflowError otherwise)."""
    v = operator.index(v)
    if v < 0:
        raise OverflowError(f"can't convert negative int to unsigned ({name})")
    if v > 0xFFFFFFFFFFFFFFFF:
        raise OverflowError(f"int too big to convert ({name})")
    return v


def _f64(v) -> float:
    return float(v)


def _bool(v, name: str) -> bool:
    if isinstance(v, (bool, np.bool_)):
        return bool(v)
    raise TypeError(f"'{type(v).__name__}' object cannot be converted to 'PyBool' ({name})")


def _as_f64_array(obj) -> np.ndarray:
    """lib.rs:25-38."""
    if not isinstance(obj, np.ndarray):
        raise TypeError(f"expected a numpy.ndarray, got {type(obj).__name__}")
    if obj.dtype != np.float64:
        obj = obj.astype("float64")
    return obj


def _as_points(obj, what: str, allow_single: bool):
    """lib.rs:54-72: returns (row-major float64 2-D array, single)."""
    a = _as_f64_array(obj)
    if a.ndim == 1 and allow_single:
        return np.ascontiguousarray(a).reshape(1, -1), True
    if a.ndim == 2:
        return np.ascontiguousarray(a), False
    raise ValueError(what)


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _result_array(shape, dtype) -> np.ndarray:
    """A fresh numpy array for query results, backed by a page-locked block
    from the engine's pool (kd_host_alloc): the kernel writes result rows
    straight into it.  The block goes back to the pool when the array (and
    every view of it) is gone.  Plain numpy memory if pinning fails."""
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    p = ctypes.c_void_p()
    if n == 0 or _lib.kd_host_alloc(n, ctypes.byref(p)) != KD_OK or not p.value:
        return np.empty(shape, dtype)
    buf = (ctypes.c_char * n).from_address(p.value)
    weakref.finalize(buf, _lib.kd_host_free, ctypes.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


class KDTree:
    """kd-tree for exact k-nearest-neighbour queries, built and queried on the GPU.

    Same surface as the reference's `kdtree.KDTree` (python/kdtree/_core.pyi).
    """

    __slots__ = ("_h", "_ndim", "_n", "_leafsize", "__weakref__")

    def __init__(self, data, *, leafsize: int = 32, parallel: bool = False):
        pts, _ = _as_points(data, "data must be a two-dimensional array", False)
        leafsize = _usize(leafsize, "leafsize")
        parallel = _bool(parallel, "parallel")
        h = ctypes.c_void_p()
        st = _lib.kd_build(_ptr(pts), pts.size, pts.shape[1], leafsize, int(parallel), ctypes.byref(h))
        if st != KD_OK:
            _raise(st)
        object.__setattr__(self, "_h", h)
        object.__setattr__(self, "_ndim", int(_lib.kd_ndim(h)))
        object.__setattr__(self, "_n", int(_lib.kd_n_points(h)))
        object.__setattr__(self, "_leafsize", int(_lib.kd_leafsize(h)))

    def __setattr__(self, name, value):
        raise AttributeError(f"'KDTree' object attribute '{name}' is read-only")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.kd_free(h)

    @property
    def ndim(self) -> int:
        return self._ndim

    @property
    def n_points(self) -> int:
        return self._n

    @property
    def leafsize(self) -> int:
        return self._leafsize

    @property
    def data(self) -> np.ndarray:
        """The points in the caller's original order (tree.rs:60-68)."""
        out = np.empty((self._n, self._ndim), np.float64)
        st = _lib.kd_original_data(self._h, _ptr(out))
        if st != KD_OK:
            _raise(st)
        return out

    def __len__(self) -> int:
        return self._n

    def __repr__(self) -> str:
        return f"KDTree(n_points={self._n}, ndim={self._ndim}, leafsize={self._leafsize})"

    def query(self, x, *, k: int = 1, p: float = 2.0, max_distance: float | None = None, eps: float = 0.0,
              parallel: bool = False):
        """Exact k nearest neighbours of each row of `x` (lib.rs:161-182)."""
        q, single = _as_points(x, "query must be one- or two-dimensional", True)
        if q.shape[1] != self._ndim:
            raise ValueError(f"dimension mismatch: expected {self._ndim}, got {q.shape[1]}")
        k = _usize(k, "k")
        p = _f64(p)
        has_max = max_distance is not None
        md = _f64(max_distance) if has_max else 0.0
        eps = _f64(eps)
        parallel = _bool(parallel, "parallel")
        nq = q.shape[0]
        if k == 0 or nq == 0:
            # validation errors; the engine reports them without touching outputs
            dummy_d = np.empty(1, np.float64)
            dummy_i = np.empty(1, np.int64)
            st = _lib.kd_query(self._h, _ptr(q) if q.size else None, q.size, k, p, int(has_max), md, eps,
                               int(parallel), _ptr(dummy_d), _ptr(dummy_i))
            _raise(st if st != KD_OK else 10)
        out_d = _result_array((nq, k), np.float64)
        out_i = _result_array((nq, k), np.int64)
        st = _lib.kd_query(self._h, _ptr(q), q.size, k, p, int(has_max), md, eps, int(parallel), _ptr(out_d),
                           _ptr(out_i))
        if st != KD_OK:
            _raise(st)
        if single:
            return out_d[0], out_i[0]
        return out_d, out_i

    def query_async(self, queries, out_distances, out_indices, status, *, k: int = 1, p: float = 2.0,
                    max_distance: float | None = None, eps: float = 0.0, stream=None):
        """Stream-ordered query on device arrays (kd_query_async): queries
        [n, ndim] f64, out_distances [n, k] f64, out_indices [n, k] i64 and
        status (one u32 / i32) are CUDA arrays (e.g. torch tensors); returns once
        the work is enqueued on `stream` (an int handle, an object with
        `cuda_stream`, or None for the legacy default stream).  After the stream
        work, status bit 0 means a non-finite query, bit 1 a tensor-core wait
        that ran out.  Host-checkable errors raise at once."""
        iface = getattr(queries, "__cuda_array_interface__", None)
        n = int(iface["shape"][0]) if iface else 0
        k = _usize(k, "k")
        if k == 0:  # the engine's own message (InvalidK)
            one = ctypes.c_void_p(1)
            _raise(_lib.kd_query_async(self._h, one, self._ndim, 0, 2.0, 0, 0.0, 0.0, one, one, one, None))
        qa = _cuda_array(queries, "<f8", (n, self._ndim), "queries")
        da = _cuda_array(out_distances, "<f8", (n, k), "out_distances")
        ia = _cuda_array(out_indices, "<i8", (n, k), "out_indices")
        siface = getattr(status, "__cuda_array_interface__", None)
        if siface is None or siface["typestr"] not in ("<u4", "<i4"):
            raise TypeError("status: expected a 4-byte integer CUDA array")
        has_max = max_distance is not None
        s = getattr(stream, "cuda_stream", stream)
        st = _lib.kd_query_async(self._h, ctypes.c_void_p(qa), n * self._ndim, k, _f64(p), int(has_max),
                                 _f64(max_distance) if has_max else 0.0, _f64(eps), ctypes.c_void_p(da),
                                 ctypes.c_void_p(ia), ctypes.c_void_p(int(siface["data"][0])),
                                 ctypes.c_void_p(s) if s else None)
        if st != KD_OK:
            _raise(st)

    # -- inspection (no reference counterpart in Python; mirrors Tree's fields)
    def _export(self):
        """(data in tree order, indices, node words [n_nodes, 4], split values, boxes)."""
        nn = int(_lib.kd_n_nodes(self._h))
        data = np.empty((self._n, self._ndim), np.float64)
        idx = np.empty(self._n, np.uint32)
        words = np.empty((nn, 4), np.uint32)
        split = np.empty(nn, np.float64)
        boxes = np.empty((nn, 2, self._ndim), np.float64)
        st = _lib.kd_export(self._h, _ptr(data), _ptr(idx), _ptr(words), _ptr(split), _ptr(boxes))
        if st != KD_OK:
            _raise(st)
        return data, idx, words, split, boxes


# -- batched queries over many trees (no reference counterpart) -------------
class _BatchJob(ctypes.Structure):
    _fields_ = [("tree", ctypes.c_void_p), ("d_queries", ctypes.c_void_p), ("n_queries", ctypes.c_uint64),
                ("k", ctypes.c_uint64), ("d_out_distances", ctypes.c_void_p), ("d_out_indices", ctypes.c_void_p)]


BATCH_GRAPH, BATCH_FUSED, BATCH_PER_JOB = 0, 1, 2


def _cuda_array(a, typestr: str, shape, what: str) -> int:
    """Device address of a C-contiguous CUDA array (anything exposing
    __cuda_array_interface__, e.g. a torch tensor) of the given dtype and shape."""
    iface = getattr(a, "__cuda_array_interface__", None)
    if iface is None:
        raise TypeError(f"{what}: expected a CUDA device array, got {type(a).__name__}")
    if iface["typestr"] != typestr or tuple(iface["shape"]) != tuple(shape):
        raise ValueError(f"{what}: expected {typestr} of shape {tuple(shape)}, got {iface['typestr']} "
                         f"{tuple(iface['shape'])}")
    strides = iface.get("strides")
    if strides is not None:
        item = int(typestr[2:])
        want, acc = [], item
        for n in reversed(shape):
            want.append(acc)
            acc *= n
        if tuple(strides) != tuple(reversed(want)):
            raise ValueError(f"{what}: must be C-contiguous")
    return int(iface["data"][0])


class BatchQuery:
    """Exact k-NN for many (tree, query batch) jobs in one pass on the device
    (kd_batch_* in include/kdtree_gb300.h).  No reference counterpart: it fuses
    a caller's loop of `KDTree.query` calls; each job's results equal that
    call's.  Jobs are (tree, queries[n, ndim] f64, k, out_distances[n, k] f64,
    out_indices[n, k] i64), arrays in device memory that stay valid while the
    plan lives; `run()` recomputes every job from the arrays' current contents.
    """

    __slots__ = ("_h", "_trees")

    def __init__(self, jobs, *, p: float = 2.0, max_distance=None, eps: float = 0.0):
        jobs = list(jobs)
        arr = (_BatchJob * max(len(jobs), 1))()
        for j, (tree, q, k, od, oi) in enumerate(jobs):
            if not isinstance(tree, KDTree):
                raise TypeError(f"job {j}: expected a KDTree")
            k = _usize(k, "k")
            n = int(q.__cuda_array_interface__["shape"][0]) if hasattr(q, "__cuda_array_interface__") else 0
            arr[j] = _BatchJob(tree._h, _cuda_array(q, "<f8", (n, tree.ndim), f"job {j} queries"), n, k,
                               _cuda_array(od, "<f8", (n, k), f"job {j} distances"),
                               _cuda_array(oi, "<i8", (n, k), f"job {j} indices"))
        h = ctypes.c_void_p()
        has_max = max_distance is not None
        st = _lib.kd_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(jobs), _f64(p), int(has_max),
                                  _f64(max_distance) if has_max else 0.0, _f64(eps), ctypes.byref(h))
        if st != KD_OK:
            _raise(st)
        self._h = h
        self._trees = [j[0] for j in jobs]  # keep the trees alive with the plan

    def run(self, stream=None, mode: int = BATCH_GRAPH):
        """Run every job on `stream` (a CUDA stream handle as an int, or an
        object with a `cuda_stream` attribute; None = the legacy default
        stream) and wait for it."""
        s = getattr(stream, "cuda_stream", stream)
        st = _lib.kd_batch_run_mode(self._h, ctypes.c_void_p(s) if s else None, int(mode))
        if st != KD_OK:
            _raise(st)

    def choice(self) -> dict:
        """The autotuner's choice (kd_batch_choice): persistent grid in CTAs,
        sorting by landing leaf, and the widths whose k <= 4 jobs run as
        packet tasks."""
        blocks, srt, pw = ctypes.c_uint(), ctypes.c_int(), ctypes.c_uint()
        st = _lib.kd_batch_choice(self._h, ctypes.byref(blocks), ctypes.byref(srt), ctypes.byref(pw))
        if st != KD_OK:
            _raise(st)
        return {"blocks": blocks.value, "sorted": bool(srt.value),
                "packet_widths": [w for b, w in enumerate((2, 3, 8)) if (pw.value >> b) & 1]}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.kd_batch_free(h)
            self._h = None


# -- serving loop (no reference counterpart) ---------------------------------
class Server:
    """Continuous-batching query server over a fixed list of trees
    (kd_server_* in include/kdtree_gb300.h).  `submit` queues a request and
    returns a ticket at once; `wait` returns (distances, indices, latency_s),
    the results exactly those of `trees[tree].query(queries, k=k, ...)`.
    No reference counterpart: it is a request loop in front of KDTree.query."""

    __slots__ = ("_h", "_trees", "_pending", "__weakref__")

    def __init__(self, trees, *, p: float = 2.0, max_distance=None, eps: float = 0.0, max_batch_queries: int = 0):
        trees = list(trees)
        for i, t in enumerate(trees):
            if not isinstance(t, KDTree):
                raise TypeError(f"tree {i}: expected a KDTree")
        arr = (ctypes.c_void_p * max(len(trees), 1))(*[t._h for t in trees])
        h = ctypes.c_void_p()
        has_max = max_distance is not None
        st = _lib.kd_server_create(ctypes.cast(arr, ctypes.c_void_p), len(trees), _f64(p), int(has_max),
                                   _f64(max_distance) if has_max else 0.0, _f64(eps),
                                   _usize(max_batch_queries, "max_batch_queries"), ctypes.byref(h))
        if st != KD_OK:
            _raise(st)
        self._h = h
        self._trees = trees
        self._pending = {}

    def submit(self, tree: int, queries, k: int, out=None) -> int:
        """Queue `queries` (2-D, tree's width) against trees[tree]; `out` may be
        a preallocated (float64 [n, k], int64 [n, k]) pair, e.g. page-locked."""
        t = self._trees[tree]
        q, _ = _as_points(queries, "query must be one- or two-dimensional", True)
        if q.shape[1] != t.ndim:
            raise ValueError(f"dimension mismatch: expected {t.ndim}, got {q.shape[1]}")
        k = _usize(k, "k")
        n = q.shape[0]
        if out is None:
            out = (_result_array((n, k), np.float64), _result_array((n, k), np.int64))
        od, oi = out
        if od.shape != (n, k) or oi.shape != (n, k) or od.dtype != np.float64 or oi.dtype != np.int64 \
                or not od.flags.c_contiguous or not oi.flags.c_contiguous:
            raise ValueError("out must be C-contiguous float64 and int64 arrays of shape (n, k)")
        ticket = ctypes.c_uint64()
        st = _lib.kd_server_submit(self._h, tree, _ptr(q) if q.size else None, n, k, _ptr(od) if od.size else None,
                                   _ptr(oi) if oi.size else None, ctypes.byref(ticket))
        if st != KD_OK:
            _raise(st)
        self._pending[ticket.value] = (q, od, oi)
        return ticket.value

    def wait(self, ticket: int):
        lat = ctypes.c_double()
        st = _lib.kd_server_wait(self._h, ticket, ctypes.byref(lat))
        entry = self._pending.pop(ticket, None)
        if st != KD_OK:
            _raise(st)
        return entry[1], entry[2], lat.value

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.kd_server_free(h)
            self._h = None
            self._pending.clear()

    def __del__(self):
        self.close()
