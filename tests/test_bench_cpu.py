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
