"""The C-ABI library without a GPU: it loads, exports every declared symbol, and
the host-side validation reports the reference's statuses and messages
(src/build.rs:25-43, src/error.rs:18-51) before any device work.  The Python
boundary's own checks (src/lib.rs:25-84) are covered here too."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "kdtree_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(kd_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    import build_lib

    L = ctypes.CDLL(str(build_lib.LIB))
    L.kd_build.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_void_p)]
    L.kd_build.restype = ctypes.c_int
    L.kd_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.kd_last_error.restype = ctypes.c_size_t
    L.kd_count_nodes.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    L.kd_count_nodes.restype = ctypes.c_uint64
    return L


def last_error(L):
    buf = ctypes.create_string_buffer(512)
    L.kd_last_error(buf, 512)
    return buf.value.decode()


def test_header_declares_the_reference_entry_points():
    syms = declared_symbols()
    for s in ("kd_build", "kd_query", "kd_free", "kd_original_data", "kd_last_error", "kd_query_device",
              "kd_build_device", "kd_export", "kd_count_nodes", "kd_query_async"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def _build(lib, data_ptr, n_values, ndim, leafsize):
    out = ctypes.c_void_p()
    st = lib.kd_build(data_ptr, n_values, ndim, leafsize, 0, ctypes.byref(out))
    return st, last_error(lib)


def test_build_validation_order_and_messages(lib):
    dummy = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    assert _build(lib, dummy, 6, 2, 0) == (2, "leafsize must be greater than zero")
    assert _build(lib, dummy, 0, 2, 32) == (1, "data must contain at least one point")
    assert _build(lib, dummy, 6, 0, 32) == (1, "data must contain at least one point")
    assert _build(lib, dummy, 7, 2, 32) == (10, "data length must be a multiple of ndim")
    n = 2**32
    assert _build(lib, dummy, n, 1, 32) == (8, f"n_points must fit in a 32-bit index, got {n}")
    n = 2**32 - 1
    st, msg = _build(lib, dummy, n, 1, 1)
    assert st == 9
    assert msg == (f"tree would need {2 * n - 1} nodes, which exceeds the 32-bit node index; "
                   "increase leafsize")


def test_count_nodes_matches_oracle(lib, oracle):
    for n in (1, 2, 17, 100, 1000, 10_000, 1_000_000, 2**32 - 1):
        for ls in (1, 6, 16, 32):
            assert lib.kd_count_nodes(n, ls) == oracle.count_nodes(n, ls)


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="only meaningful without a GPU")
def test_no_cpu_fallback(lib):
    data = np.zeros((4, 2))
    st, msg = _build(lib, ctypes.c_void_p(data.ctypes.data), 8, 2, 32)
    assert st == 103 and "no CPU fallback" in msg


def test_python_boundary_checks_before_native_work():
    from kdtree import KDTree

    with pytest.raises(TypeError, match="expected a numpy.ndarray"):
        KDTree([[0.0, 1.0]])
    with pytest.raises(ValueError, match="data must be a two-dimensional array"):
        KDTree(np.zeros((2, 2, 2)))
    with pytest.raises(ValueError, match="data must be a two-dimensional array"):
        KDTree(np.zeros(3))
    with pytest.raises(ValueError, match="data must contain at least one point"):
        KDTree(np.zeros((0, 3)))
    with pytest.raises(ValueError, match="leafsize must be greater than zero"):
        KDTree(np.zeros((3, 3)), leafsize=0)
    with pytest.raises(OverflowError):
        KDTree(np.zeros((3, 3)), leafsize=-1)
    with pytest.raises(TypeError):
        KDTree(np.zeros((3, 3)), leafsize=1.5)
