"""Type switch moves on the GPU (MoveCreator::switchTypeMove, scOOP/mc/movecreator.cpp:233-303).

Ensemble parity: tests/golden/ens_switch_psc.json holds the energy per particle and the
switched fraction (the switched column of the reference's movie frames) of twelve runs of the
reference's own loop (oracle/_ref/sc_ref, tests/golden/make_ensemble.py): 150 PSC particles
whose type switches to a CPSC type and back with delta_mu = 1.6 (the reference reads it
into an int: 1), beside 50 fixed spheres, switchprob 0.1.  As many GPU trajectories from
the same start as the reference ran; both means within 2 combined standard errors.

Exactness: the running energy equals the exact total after switch moves; the switched flags
follow the types; delta_mu enters as the reference's int (1.6 and 1.0 give the same run).
"""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case():
    with open(os.path.join(GOLDEN, "ens_switch_psc.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    o["paraltemper"] = o["temper"]
    return g, "".join(f"{k} = {v}\n" for k, v in o.items()), g["inputs"]["top.init"], g["inputs"]["config.init"]


def test_ensemble_matches_reference():
    from sc_gb300 import ReplicaSet, System

    g, opts, top, cfg = _case()
    systems = [System.from_text(opts, top, cfg) for _ in range(g["seeds"])]
    T = float(g["options"]["temper"])
    R = ReplicaSet(systems, [T] * len(systems), ladder=list(range(len(systems))))
    p = systems[0].default_run()
    p.check_every = 0
    assert p.switchprob == 0.1
    rep, burn, nsw = g["report"], g["burn"], g["nsweeps"]
    E = [[] for _ in systems]
    F = [[] for _ in systems]
    done = 0
    while done < nsw:
        _, _, en, _, _ = R.run(rep, exchange_every=0, seed=4242, params=p)
        done += rep
        if done > burn:
            for k, s in enumerate(systems):
                E[k].append(en[k] / s.n)
                F[k].append(sum(1 for q in s.particles(0, 150) if q.type == 2) / 150.0)
    R.close()
    for s in systems:
        exact = s.all_to_all()
        st = s.simulate(p, nsweeps=0)
        assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact))
        s.close()
    report = {}
    for key, ser in (("energy_per_particle", E), ("switched_fraction", F)):
        m = np.array([np.mean(x) for x in ser])
        mean, se = float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))
        ref = g["stats"][key]
        report[key] = (mean, se, ref["mean"], ref["se"])
    print("switch ensemble (GPU mean, se, reference mean, se):", report)
    for key, (mean, se, rm, rse) in report.items():
        assert abs(mean - rm) <= 2.0 * math.sqrt(se ** 2 + rse ** 2), report


def test_running_energy_exact_and_flags_follow_types(tmp_path):
    from sc_gb300 import System

    g, opts, top, cfg = _case()
    s = System.from_text(opts, top, cfg)
    p = s.default_run()
    p.check_every = 0
    p.seed = 5
    st = s.simulate(p, nsweeps=300)
    assert st.acc_switch > 0 and st.rej_switch > 0
    exact = s.all_to_all()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
    s.write_config(str(tmp_path / "c"))
    rows = (tmp_path / "c").read_text().splitlines()[1:]
    types = [q.type for q in s.particles()]
    for k in range(150):
        assert int(rows[k].split()[9]) == (1 if types[k] == 2 else 0)
    assert all(t == 3 for t in types[150:])
    s.close()


def test_delta_mu_is_read_as_an_int():
    from sc_gb300 import System

    g, opts, top, cfg = _case()
    out = []
    for dmu in ("1.6", "1.0"):
        s = System.from_text(opts, top.replace("particles: 1 2 1.6", f"particles: 1 2 {dmu}"), cfg)
        p = s.default_run()
        p.seed = 77
        st = s.simulate(p, nsweeps=200)
        out.append((st.energy, st.acc_switch, [q.type for q in s.particles()]))
        s.close()
    assert out[0] == out[1]
