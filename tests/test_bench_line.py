"""Host-side pieces of the bench line (no GPU): the roofline's algorithmic
bytes, the ncu-measured inputs (profiles/roofline_inputs.json: DRAM traffic
with its commit and a staleness check against the kernel sources), the
measured peak, and the build's level count and bytes."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_algorithmic_bytes_formula():
    # B_q = 8d + 16k + 8d*S_q + 24*V_q + 16d*X_q, summed: one query, 2 nodes, 5 rows, 1 box
    d, k = bench.DIM, bench.K
    assert bench.algorithmic_bytes((2, 5, 1), 1) == 8 * d + 16 * k + 8 * d * 5 + 24 * 2 + 16 * d * 1


def test_profiled_inputs_carry_their_commit_and_staleness():
    j = bench.profiled_inputs()
    pk = j["k_query_packet"]
    t = pk["traffic_bytes_per_launch"]
    assert isinstance(t, int) and t == pk["dram_read_bytes"] + pk["dram_write_bytes"] > 0
    assert j["commit"] and isinstance(pk["stale"], bool) and 0 < pk["l2_hit_rate_pct"] <= 100
    assert all((ROOT / f).exists() for f in pk["source_files"])
    assert 0 < j["build"]["l2_hit_rate_pct_time_weighted"] <= 100
    # the summary of the same capture states the same traffic
    text = (ROOT / "profiles" / "k_query_packet_uniform_n1m_d3_k16.md").read_text()
    assert "126.4 MB / 216.0 MB" in text


def test_measured_peak_is_positive():
    peak, kind = bench.measured_peak()
    assert peak > 0 and kind in ("measured", "fallback")


def test_build_line_levels_and_bytes():
    b = bench.build_line(0.005, 0.04, 6000.0)
    # 1M rows, leafsize 16: segments of ceil(1M / 2^t) rows split while above 16 -> 16 levels
    assert b["levels"] == 16
    assert b["algorithmic_bytes"] == 16 * bench.N_POINTS * (3 * 8 * bench.DIM + 8)
    assert abs(b["achieved_gbs"] - b["algorithmic_bytes"] / 0.005 / 1e9) < 1e-6
    assert b["frac_of_hbm"] == b["achieved_gbs"] / 6000.0
    assert bench.build_line(0.005, None, None)["frac_of_hbm"] is None


def test_scipy_baseline_small():
    import numpy as np
    import pytest

    pytest.importorskip("scipy")
    rng = np.random.default_rng(0)
    r = bench.scipy_baseline(rng.uniform(size=(2000, 3)), rng.uniform(size=(300, 3)), k=4, leafsize=16)
    assert r["qps"] > 0 and r["build_s"] >= 0 and r["workers"] >= 1


def test_count_nodes_matches_the_reference_sizes():
    # the node counts the reference's layout gives (N=1M leafsize 16, N=10k leafsize 32)
    assert bench.count_nodes(1_000_000, 16) == 131_071
    assert bench.count_nodes(10_000, 32) == 1_023
    assert bench.count_nodes(5, 32) == 1


def test_compulsory_bytes_close_to_profiled_traffic():
    c = bench.compulsory_bytes()
    # queries 24 MB + results 256 MB + the tree once
    assert c > bench.N_QUERIES * (bench.DIM * 8 + bench.K * 16)
    t = bench.profiled_inputs()["k_query_packet"]["traffic_bytes_per_launch"]
    assert 0.5 < t / c < 2.0
