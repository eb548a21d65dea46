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
