"""The output files of the move loop in the reference's formats (energy.dat, stat.dat, movie,
config.last) and the alignment order (Updater::alignmentOrder) on the GPU."""
import os

import numpy as np
import pytest

from test_gpu_sweep import alignment_order, open_ens

pytestmark = pytest.mark.gpu


def test_alignment_order_matches_pair_sum():
    _, s = open_ens("psc_nvt")
    s.simulate(nsweeps=20, seed=3, check_every=0)
    assert abs(s.alignment_order() - alignment_order(s)) <= 1e-9 * max(1.0, abs(alignment_order(s)))
    s.close()


def test_run_writes_the_reference_files(tmp_path):
    from sc_gb300 import System, updater

    _, s = open_ens("cpsc_spa_npt")
    totals = updater.run(s, 60, report=20, movie=30, directory=str(tmp_path), seed=4, check_every=0)
    assert totals["moves"] == 60 * s.n
    e = [l for l in open(tmp_path / "energy.dat") if not l.startswith("#")]
    v = [l for l in open(tmp_path / "stat.dat") if not l.startswith("#")]
    assert [int(l.split(";")[0]) for l in e] == [20, 40, 60] and len(v) == 3
    en, al = (float(x) for x in e[-1].split(";")[1].split())
    assert abs(en - s.all_to_all()) <= 1e-9 * abs(en) and abs(al - alignment_order(s)) < 1e-5
    assert abs(float(v[-1].split(";")[1]) - np.prod(s.box)) < 1e-8 * np.prod(s.box)
    movie = open(tmp_path / "movie").read().splitlines()
    assert len(movie) == 2 * (s.n + 2) and movie[1].startswith("sweep 30; box ")
    assert len(movie[2].split()) == 11
    last = open(tmp_path / "config.last").read().splitlines()
    assert len(last) >= s.n + 1
    s.close()


def test_run_writes_the_wang_landau_file_and_stops_where_the_reference_stops(tmp_path):
    import gzip
    import json

    from sc_gb300 import System, updater

    here = os.path.dirname(os.path.abspath(__file__))
    with gzip.open(os.path.join(here, "golden", "wl", "cases.json.gz"), "rt") as f:
        c = {c["name"]: c for c in json.load(f)["cases"]}["o4_pair"]
    inp = c["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    lines = inp["wl.dat"].splitlines()
    # alpha below WL_ALPHATOL, a histogram flat at the first check: the run ends at sweep 1000
    s.wl_load(text="5e-9\n" + "".join(f"{l.split()[0]} 0.0 1000000000\n" for l in lines[1:]))
    totals = updater.run(s, 3000, report=500, directory=str(tmp_path), seed=5, variant=4)
    assert totals["sweeps"] == 1000 and totals["moves"] == 1000 * s.n
    e = [l for l in open(tmp_path / "energy.dat") if not l.startswith("#")]
    assert [int(l.split(";")[0]) for l in e] == [500, 1000]
    wl = open(tmp_path / "wl-new.dat").read().splitlines()
    assert wl[0].strip() == "5.00000000e-09" and len(wl) == 1 + len(lines) - 1
    s.close()
