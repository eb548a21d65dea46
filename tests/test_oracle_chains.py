"""The oracle's chain moves (MoveCreator::chainMove, chainDisplace, chainRotate, clusterRotate;
scOOP/mc/movecreator.cpp:305-328, 1075-1392) in its sequential loop, on the CPU.

- Rigid moves: the bonds inside every chain keep their lengths (to rounding), the running
  energy equals a fresh total after many chain and particle moves, with the energy matrix
  and without it, with the pair list and without it.
- The ensemble of 64 three-bead lipids with chain moves (tests/golden/ens_lipids_chain.json:
  the reference's own loop, oracle/_ref/sc_ref, six seeds of 30,000 sweeps): four oracle runs
  of 6000 sweeps give its mean energy per particle within three combined standard errors.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle_ffi import McRun, TextSystem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _lipids():
    with open(os.path.join(GOLDEN, "ens_lipids_chain.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    return g, o, g["inputs"]["top.init"], g["inputs"]["config.init"]


def _text(o):
    return "".join(f"{k} = {v}\n" for k, v in o.items())


def _bond_lengths(ts):
    box = np.array(list(ts.sys.box))
    pos = np.array([[p.pos.x, p.pos.y, p.pos.z] for p in ts.parts[: ts.sys.n]])
    out = []
    for c in range(ts.sys.n // 3):
        for a, b in ((0, 1), (1, 2)):
            d = pos[3 * c + a] - pos[3 * c + b]
            d = (d - np.rint(d)) * box
            out.append(np.linalg.norm(d))
    return np.array(out)


@pytest.mark.parametrize("matrix", [True, False])
@pytest.mark.parametrize("plist", [10, 0])
def test_chain_moves_are_rigid_and_keep_the_energy_exact(matrix, plist):
    g, o, top, cfg = _lipids()
    o = dict(o, pairlist_update=plist, chainprob=0.5)
    ts = TextSystem(_text(o), top, cfg)
    b0 = _bond_lengths(ts)
    pos0 = np.array([[p.pos.x, p.pos.y, p.pos.z] for p in ts.parts[: ts.sys.n]])
    run = McRun(ts, seed=3, energy_matrix=matrix)
    run.sweeps(15)
    st = run.stats
    assert st.acc_chain > 50 and st.rej_chain > 0, (st.acc_chain, st.rej_chain)
    assert st.acc_trans + st.acc_rot > 0
    exact = ts.all_to_all()
    assert abs(run.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (run.energy, exact)
    run.close()
    # chain moves alone move the chains rigidly: every bond keeps its length
    o1 = dict(o, chainprob=1.0)
    ts = TextSystem(_text(o1), top, cfg)
    run = McRun(ts, seed=4, energy_matrix=matrix)
    run.sweeps(8)
    assert run.stats.acc_chain > 50
    assert run.stats.acc_trans + run.stats.rej_trans + run.stats.acc_rot + run.stats.rej_rot == 0
    assert np.allclose(_bond_lengths(ts), b0, rtol=0, atol=1e-9)
    pos1 = np.array([[p.pos.x, p.pos.y, p.pos.z] for p in ts.parts[: ts.sys.n]])
    assert not np.allclose(pos1, pos0)
    exact = ts.all_to_all()
    assert abs(run.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (run.energy, exact)
    run.close()


def _ensemble_run(seed, nsw=6000, burn=2000):
    """Mean energy per particle of one oracle run (the -Ofast build of the same restatement)."""
    g, o, top, cfg = _lipids()
    n, rep = g["n"], g["report"]
    ts = TextSystem(_text(o), top, cfg)
    r = McRun(ts, seed=seed, fast=True)
    e = []
    for k in range(rep, nsw + 1, rep):
        r.sweeps(rep)
        if k > burn:
            e.append(r.energy / n)
    chains = r.stats.acc_chain
    r.close()
    return float(np.mean(e)), int(chains)


def test_ensemble_matches_reference():
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    g = _lipids()[0]
    with ProcessPoolExecutor(max_workers=4, mp_context=mp.get_context("spawn")) as ex:
        runs = list(ex.map(_ensemble_run, range(1, 5)))
    assert all(c > 0 for _, c in runs)
    m = np.array([e for e, _ in runs])
    mean, se = float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))
    ref = g["stats"]["energy_per_particle"]
    report = (mean, se, ref["mean"], ref["se"])
    print("oracle lipid chain ensemble (mean, se, reference mean, se):", report)
    assert abs(mean - ref["mean"]) <= 3.0 * math.sqrt(se ** 2 + ref["se"] ** 2), report
