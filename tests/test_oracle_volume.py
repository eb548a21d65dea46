"""The oracle's volume move for every coupling of MoveCreator::pressureMove
(scOOP/mc/movecreator.cpp:349-546) on the CPU.

- What each coupling keeps: ptype 2 and 4 keep z, 4 and 5 keep the other edges, 3 keeps
  the volume (z re-derived from it) and x = y; the running energy stays exact through
  accepted and rejected moves, with the energy matrix and without it.
- Ensembles against the reference's own loop (tests/golden/ens_spa_ptype*.json: oracle/_ref/sc_ref,
  eight seeds of 20,000 sweeps of 64 attractive spheres at T = 2, P* = 1): four oracle runs
  of 5000 sweeps give the mean energy and volume per particle (for ptype 3, whose volume is
  fixed, the energy and the box x) within three combined standard errors.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle_ffi import McRun, TextSystem

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PTYPES = (0, 2, 3, 4, 5)


def _case(pt):
    with open(os.path.join(GOLDEN, f"ens_spa_ptype{pt}.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    return g, "".join(f"{k} = {v}\n" for k, v in o.items()), g["inputs"]["top.init"], g["inputs"]["config.init"]


@pytest.mark.parametrize("matrix", [True, False])
@pytest.mark.parametrize("pt", PTYPES)
def test_coupling_keeps_what_it_should(pt, matrix):
    g, opts, top, cfg = _case(pt)
    ts = TextSystem(opts, top, cfg)
    b0 = np.array(list(ts.sys.box))
    v0 = float(np.prod(b0))
    run = McRun(ts, seed=5, energy_matrix=matrix)
    seen = set()
    for _ in range(60):
        run.sweeps(10)
        b = np.array(list(ts.sys.box))
        seen.add(tuple(b))
        if pt in (2, 4):
            assert b[2] == b0[2]
        if pt == 4:
            assert b[1] == b0[1]
        if pt == 5:
            assert b[0] == b0[0] and b[2] == b0[2]
        if pt == 3:
            assert b[0] == b[1]
            assert abs(float(np.prod(b)) - v0) <= 1e-12 * v0
    st = run.stats
    assert st.acc_vol > 20 and st.rej_vol > 0, (st.acc_vol, st.rej_vol)
    assert len(seen) > 20
    if pt == 0:                       # every edge moves, each on its own
        arr = np.array(sorted(seen))
        assert all(len(set(arr[:, k])) > 5 for k in range(3))
    exact = ts.all_to_all()
    assert abs(run.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (run.energy, exact)
    run.close()


@pytest.mark.parametrize("pt", PTYPES)
def test_ensemble_matches_reference(pt):
    g, opts, top, cfg = _case(pt)
    n = g["n"]
    rep, burn, nsw = 20, 1000, 5000
    E, Vn, X = [], [], []
    for seed in range(1, 5):
        ts = TextSystem(opts, top, cfg)
        r = McRun(ts, seed=seed)
        e, v, x = [], [], []
        for k in range(rep, nsw + 1, rep):
            r.sweeps(rep)
            if k > burn:
                b = list(ts.sys.box)
                e.append(r.energy / n)
                v.append(b[0] * b[1] * b[2] / n)
                x.append(b[0])
        E.append(np.mean(e))
        Vn.append(np.mean(v))
        X.append(np.mean(x))
        r.close()
    obs = [("energy_per_particle", E)] + ([("box_x", X)] if pt == 3 else [("volume_per_particle", Vn)])
    report = {}
    for key, vals in obs:
        m = np.array(vals)
        mean, se = float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))
        ref = g["stats"][key]
        report[key] = (mean, se, ref["mean"], ref["se"])
    print(f"oracle ptype {pt} ensemble (mean, se, reference mean, se):", report)
    for key, (mean, se, rm, rse) in report.items():
        assert abs(mean - rm) <= 3.0 * math.sqrt(se ** 2 + rse ** 2), report
