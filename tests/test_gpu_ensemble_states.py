"""Ensemble parity at the benchmark's own state points, with the nematic order.

tests/golden/ens_psc_c0.json and ens_mixture_c1.json hold the averages the reference's own
loop samples (oracle/_ref/sc_ref, six seeds each, tests/golden/make_ensemble.py) at the
benchmark's state points: 1000 PSC at packing fraction 0.1 and T = 1 (NVT), and the CPSC +
SPA mixture at P* = 0.5 and T = 1 (NPT, isotropic volume moves; 500 particles), the
nematic order S2 computed from the reference's movie frames.  The GPU sampler -- plain
moves, and delayed acceptance with a trained network -- runs six trajectories from the
same start for the same sweeps; energy per particle, S2 and volume per particle must agree
within 2 combined standard errors (the means of independent trajectories).
"""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ens(name):
    with open(os.path.join(GOLDEN, f"ens_{name}.json")) as f:
        return json.load(f)


def _opts(d):
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(d)
    o["paraltemper"] = o["temper"]
    return "".join(f"{k} = {v}\n" for k, v in o.items())


def mean_se(series):
    m = np.array([x.mean() for x in series])
    return float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))


def sample(systems, g, seed, delayed=0):
    """Independent trajectories moved together as a replica batch without exchanges: the
    energy per particle, S2 and volume per particle every `report` sweeps after `burn`."""
    from sc_gb300 import ReplicaSet

    T = float(g["options"]["temper"])
    R = ReplicaSet(systems, [T] * len(systems), ladder=list(range(len(systems))))
    p = systems[0].default_run()
    p.check_every = 0
    p.delayed = delayed
    rep, burn, nsw = g["report"], g["burn"], g["nsweeps"]
    E, S, V, A = ([[] for _ in systems] for _ in range(4))
    done = 0
    while done < nsw:
        _, _, en, _, _ = R.run(rep, exchange_every=0, seed=seed, params=p)
        done += rep
        if done > burn:
            for k, s in enumerate(systems):
                E[k].append(en[k] / s.n)
                S[k].append(s.nematic_order()[0])
                V[k].append(float(np.prod(s.box)) / s.n)
                A[k].append(s.alignment_order() / s.n)
    R.close()
    return {"energy_per_particle": [np.array(x) for x in E], "nematic_s2": [np.array(x) for x in S],
            "volume_per_particle": [np.array(x) for x in V], "alignment_per_particle": [np.array(x) for x in A]}


def check(g, got, keys):
    report = {}
    for key in keys:
        m, se = mean_se(got[key])
        ref = g["stats"][key]
        sigma = math.sqrt(se ** 2 + ref["se"] ** 2)
        report[key] = (m, se, ref["mean"], ref["se"])
        assert abs(m - ref["mean"]) <= 2.0 * sigma, report
    return report


def _keys(g):
    keys = ["energy_per_particle", "nematic_s2"]
    if int(str(g["options"].get("shave", "0")).split()[0] or 0) > 0:
        keys.append("volume_per_particle")
    return keys


@pytest.mark.parametrize("name", ["psc_c0", "mixture_c1"])
def test_plain_moves_match_reference_at_benchmark_state(name):
    from sc_gb300 import System

    g = ens(name)
    systems = [System.from_text(_opts(g["options"]), g["inputs"]["top.init"], g["inputs"]["config.init"])
               for _ in range(6)]
    got = sample(systems, g, seed=2025)
    check(g, got, _keys(g))
    for s in systems:
        s.close()


@pytest.mark.parametrize("name", ["psc_c0", "mixture_c1"])
def test_delayed_acceptance_matches_reference_at_benchmark_state(name):
    """Delayed acceptance with a network trained on this system's own configurations (the
    exact FP64 stage decides every move the surrogate lets through) samples the reference's
    ensemble."""
    from sc_gb300 import Surrogate, System

    g = ens(name)
    texts = (_opts(g["options"]), g["inputs"]["top.init"], g["inputs"]["config.init"])
    train = System.from_text(*texts)
    sur = Surrogate(train, seed=3, capacity=2_000_000)
    for k in range(12):
        train.simulate(nsweeps=100, seed=7 + k, check_every=0)
        sur.collect(train)
    sur.train(epochs=6, batch=4096, lr=2e-3, warmup_steps=50, seed=3)
    systems = [System.from_text(*texts) for _ in range(6)]
    for s in systems:
        s.set_surrogate(sur)
    got = sample(systems, g, seed=3131, delayed=1)
    check(g, got, _keys(g))
    for s in systems:
        s.set_surrogate(None)
        s.close()
    sur.close()
    train.close()


def test_axial_rotations_match_reference():
    """Rotations about axes in a 40-degree cone around the particle axis (options coneAngle,
    MoveCreator::partAxialRotate) sample the reference's ensemble: 250 PSC at T = 0.6."""
    from sc_gb300 import System

    g = ens("psc_cone")
    systems = [System.from_text(_opts(g["options"]), g["inputs"]["top.init"], g["inputs"]["config.init"])
               for _ in range(6)]
    got = sample(systems, g, seed=777)
    check(g, got, ["energy_per_particle", "nematic_s2", "alignment_per_particle"])
    for s in systems:
        s.close()
