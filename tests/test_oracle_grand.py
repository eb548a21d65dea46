"""The oracle's grand-canonical move (MoveCreator::muVTMove, scOOP/mc/movecreator.cpp:797-924,
after every nGrandCanon-th sweep, scOOP/mc/updater.cpp:164-179) on the CPU.

- An ideal gas (the species' self pair excluded): the particle count is Poisson with mean
  V exp(chemPot) = V activity 0.6022137, whatever the start, an empty box included.
- The running energy and the molecule records (first / count) after many insertions and
  deletions equal a fresh calculation, with the energy matrix, without it, and with the
  pair list.
- Sixteen oracle runs from the start of tests/golden/ens_gc_spa.json (the reference's own
  loop, oracle/_ref/sc_ref, 32 seeds of 24000 sweeps), as long, give its mean energy and
  particle count within three combined standard errors.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle_ffi import McRun, TextSystem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gc_spa():
    with open(os.path.join(GOLDEN, "ens_gc_spa.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    return g, "".join(f"{k} = {v}\n" for k, v in o.items()), g["inputs"]["top.init"], g["inputs"]["config.init"]


def _ideal(n0, activity=0.1, box=8.0):
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update({"temper": 1.0, "transmx": 0.6, "rotmx": 30.0, "nGrandCanon": 1, "pairlist_update": 0})
    top = ("[Types]\nA 1 SPA 1.0 1.0 1.1225 0.5\n[Molecules]\nA: {\nparticles: 1\n"
           f"ACTIVITY: {activity}\n}}\n[System]\nA {n0}\n[EXCLUDE]\n1 1\n")
    rng = np.random.default_rng(11)
    rows = [f"{box} {box} {box}"]
    for _ in range(n0):
        p = rng.uniform(0, box, 3)
        rows.append(" ".join(f"{x:.6f}" for x in (*p, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0)) + " 0")
    return "".join(f"{k} = {v}\n" for k, v in o.items()), top, "\n".join(rows) + "\n"


def _check_records(ts):
    m = ts.mols[0]
    assert m.first == 0 and m.count == ts.sys.n
    assert all(ts.parts[i].molType == 0 and ts.parts[i].type == 1 for i in range(ts.sys.n))


@pytest.mark.parametrize("n0", [0, 60])
def test_ideal_gas_count_is_poisson(n0):
    opts, top, cfg = _ideal(n0)
    V = 8.0 ** 3
    mean_ref = V * 0.1 * 6.022137e23 * 1e-24
    samples = []
    for seed in (1, 2, 3, 4):
        ts = TextSystem(opts, top, cfg)
        assert ts.opts.n_gc == 1 and ts.opts.grand_every == 1
        r = McRun(ts, seed=seed)
        r.sweeps(400)                        # burn-in
        for _ in range(4000):
            r.sweeps(5)
            samples.append(r.n)
        st = r.stats
        assert st.acc_insert > 0 and st.acc_delete > 0 and st.rej_insert > 0 and st.rej_delete > 0
        _check_records(ts)
        r.close()
    x = np.array(samples, float).reshape(4, -1)
    # batch means: 4 seeds x 20 batches of 200 samples (1000 sweeps, well past the count's correlation time)
    b = x.reshape(80, -1).mean(axis=1)
    mean, se = float(b.mean()), float(b.std(ddof=1) / math.sqrt(len(b)))
    assert abs(mean - mean_ref) <= 4.0 * se + 1e-9, (mean, se, mean_ref)
    assert 0.8 <= float(x.var()) / mean_ref <= 1.25, (float(x.var()), mean_ref)


@pytest.mark.parametrize("matrix,plist", [(True, 0), (False, 0), (False, 5), (True, 5)])
def test_running_energy_and_records_after_gc_moves(matrix, plist):
    g, opts, top, cfg = _gc_spa()
    opts = opts.replace("pairlist_update = 0", f"pairlist_update = {plist}")
    ts = TextSystem(opts, top, cfg)
    r = McRun(ts, seed=9, energy_matrix=matrix)
    st = r.sweeps(600)
    assert st.acc_insert > 0 and st.acc_delete > 0
    assert ts.sys.n != 30
    _check_records(ts)
    exact = ts.all_to_all()
    assert abs(r.energy - exact) <= 1e-8 * max(1.0, abs(exact)), (r.energy, exact)
    r.close()


def test_sweep_counting_matches_or_mc_run():
    """or_mc_sweeps in blocks gives the same run as one call: the move after a sweep does
    not depend on how the steps were split."""
    g, opts, top, cfg = _gc_spa()
    out = []
    for blocks in ((300,), (1, 99, 150, 50), (7,) * 42 + (6,)):
        ts = TextSystem(opts, top, cfg)
        r = McRun(ts, seed=4)
        for b in blocks:
            r.sweeps(b)
        out.append((ts.sys.n, r.energy, r.stats.acc_insert, r.stats.acc_delete))
        r.close()
    assert out[0] == out[1] == out[2]


def test_ensemble_matches_reference():
    g, opts, top, cfg = _gc_spa()
    rep, burn, nsw = g["report"], g["burn"], g["nsweeps"]
    E, Nn = [], []
    for seed in range(1, 17):
        ts = TextSystem(opts, top, cfg)
        r = McRun(ts, seed=seed)
        e, n = [], []
        for k in range(rep, nsw + 1, rep):
            r.sweeps(rep)
            if k > burn:
                e.append(r.energy)
                n.append(r.n)
        E.append(np.mean(e))
        Nn.append(np.mean(n))
        r.close()
    report = {}
    for key, m in (("energy_total", np.array(E)), ("particles", np.array(Nn))):
        mean, se = float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))
        ref = g["stats"][key]
        report[key] = (mean, se, ref["mean"], ref["se"])
    print("oracle muVT ensemble (mean, se, reference mean, se):", report)
    for key, (mean, se, rm, rse) in report.items():
        assert abs(mean - rm) <= 3.0 * math.sqrt(se ** 2 + rse ** 2), report


def test_refuses_gc_with_switching():
    g, opts, top, cfg = _gc_spa()
    ts = TextSystem(opts + "switchprob = 0.1\n", top, cfg)
    with pytest.raises(ValueError):
        McRun(ts, seed=1)
