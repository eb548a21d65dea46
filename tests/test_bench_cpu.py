"""The CPU legs of bench.py, which time the reference's loop (the oracle's -Ofast
restatement) beside the device numbers: each runs here on small samples and returns a
positive rate for the moves it counted.  The GPU sections around them run on the GPU host."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from sc_gb300 import workloads  # noqa: E402


def test_replicas_cpu_baseline_on_two_ladders():
    systems, temps = workloads.pt_ladders(seed=1)
    r = bench.replicas_cpu_baseline(systems[:2], temps, seed=3, seconds=0.5)
    assert r["value"] > 0 and r["cores"] == 1 and r["kind"] == "port"
    n = sum(t[2].count("\n") - 1 for t in systems[:2])
    moves = int(r["sample"].split()[0])
    assert moves >= n


def test_wang_landau_cpu_baseline():
    opts, top, cfg, wl = workloads.protein_bilayer(seed=1, wlm=(1, 3), chainprob=0.0)
    rate, moves = bench.wl_cpu_baseline((opts, top, cfg), wl, 1, max_moves=300)
    assert moves == 300 and rate > 0


def test_bilayer_cpu_baseline_on_a_small_bilayer():
    r = bench.bilayer_cpu_baseline(workloads.bilayers(6, seed=2), seed=3, seconds=0.3)
    assert r["value"] > 0 and r["cores"] == 1
    words = r["sample"].split()
    moves, chains = int(words[0]), int(words[2].lstrip("("))
    assert moves >= 2000 and chains > 0


def test_roofline_arithmetic():
    """achieved = algorithmic bytes per launch / average launch time; frac = achieved / the
    measured peak; the dominant kernel is named from the launch shape, and its DRAM traffic is
    read from the committed ncu summary of that kernel and workload."""
    tot = {"phase_n": 10, "phase_s": 0.05, "tested": 1_000_000, "evaluated": 30_000}
    peaks = {"hbm_gbs": 6765.7}
    roof, fp = bench.roofline(tot, 8, "psc_cpsc_65536", peaks, "measured", None)
    per_launch = (1_000_000 * 28 + 30_000 * 120) / 10
    assert roof["kernel"] == "kCellWarpsFlow" and roof["unit"] == "GB/s" and roof["bound"] == "hbm"
    assert abs(roof["algorithmic_bytes_per_launch"] - per_launch) < 1e-6
    assert abs(roof["achieved"] - per_launch / 0.005 / 1e9) < 1e-9
    assert abs(roof["frac"] - roof["achieved"] / 6765.7) < 1e-15
    assert abs(roof["avg_launch_us"] - 5000.0) < 1e-9
    assert abs(fp["achieved_ops_per_s"] - (1_000_000 * 17 + 30_000 * 600) / 10 / 0.005) < 1e-3
    fp64 = {"dmul_dadd_ops_per_s": 5.29e11, "dfma_flops": 1.26e12, "one_lane_ops_per_s": 1.6e10,
            "latency_cycles": 64.0}
    _, fp = bench.roofline(tot, 8, "psc_cpsc_65536", peaks, "measured", fp64)
    assert abs(fp["frac"] - fp["achieved_ops_per_s"] / 5.29e11) < 1e-15
