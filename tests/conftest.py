"""Test configuration: import paths, the `gpu` marker, and on-demand builds.

`-m "not gpu"` runs on any machine (oracle against the golden fixtures and
SciPy, C-ABI exports and host-side validation).  `-m gpu` needs a CUDA GPU and
compares the GPU engine with the oracle through the C ABI.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "tests" / "golden", ROOT / "oracle", ROOT / "kdtree-rs_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine")
    # Build the checker and the engine once, before any test imports them.
    import kdtree_oracle

    kdtree_oracle.build_oracle()
    import build_lib

    build_lib.build()


@pytest.fixture(scope="session")
def oracle():
    import kdtree_oracle

    return kdtree_oracle
