"""Compile libkdtree_gb300.so (the CUDA engine behind include/kdtree_gb300.h).

Each translation unit is compiled for sm_103a in parallel, then linked into one
shared library in `_build/` next to this file.  Usable as a script
(`python kdtree-rs_gb300/build_lib.py`) or through `build()`.

`build(counting=True)` makes a measurement variant, `_build/counts/
libkdtree_gb300_counts.so`, compiled with KD_WORK_COUNTS: the packet traversal
then counts the work it does (nodes, leaves, rows, offers) in device counters
that kd_work_counts reads.  The product library never has them.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libkdtree_gb300.so"
SOURCES = ["kd_api.cu", "kd_build.cu", "kd_query.cu", "kd_query_tc.cu", "kd_noalloc.cu", "kd_batch.cu",
           "kd_query_packet.cu", "kd_query_warp.cu", "kd_query_ref.cu"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    # Every FP64 result that must equal the reference's is written with explicit
    # round-to-nearest intrinsics; -fmad=false keeps the compiler from fusing any
    # remaining multiply-add as well (rustc never contracts).
    "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "-Xptxas", "-O3",
]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src, *CSRC.glob("*.cuh"), *CSRC.glob("*.hpp"), HERE.parent / "include" / "kdtree_gb300.h",
            Path(__file__)]
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False, counting: bool = False) -> Path:
    out = OUT / "counts" if counting else OUT
    lib = out / "libkdtree_gb300_counts.so" if counting else LIB
    flags = [*NVCC_FLAGS, "-DKD_WORK_COUNTS"] if counting else NVCC_FLAGS
    out.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for s in SOURCES:
        src = CSRC / s
        obj = out / (s + ".o")
        if force or _stale(obj, src):
            jobs.append([nvcc, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    objs = [str(out / (s + ".o")) for s in SOURCES]
    if jobs or not lib.exists():
        tmp = out / (lib.name + ".tmp")
        run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", str(tmp), "-lcudart"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(p)
