"""The multi-GPU path is replicas only: every rank holds the tree and queries
its own batch, with no collective on the data path.  Its host-side logic --
per-rank query seeds, the whole-job rate over the slowest rank -- runs here on
two CPU processes over gloo (127.0.0.1)."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    got_ws, got_rank, _ = bench.dist_env()
    rate, slowest = bench.whole_job_rate(1.0 + rank, 2, got_ws, "cpu")
    data, q = bench.workload(got_rank)
    np.save(out / f"r{rank}.npy", np.array([rate, slowest, q[0, 0], data[0, 0], got_rank, got_ws]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_over_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ws, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(ws, port, tmp_path), nprocs=ws, start_method="spawn", join=True)
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    # max over ranks: both see the slowest rank's 2.0 s; 2 ranks x 2 steps x 10^6 queries
    assert r0[1] == r1[1] == 2.0
    assert r0[0] == r1[0] == 2 * 2 * 1_000_000 / 2.0
    # the same tree on every rank, each rank its own queries
    assert r0[3] == r1[3] and r0[2] != r1[2]
    assert (r0[4], r1[4], r0[5]) == (0, 1, 2)
