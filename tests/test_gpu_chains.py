"""Chain moves (MoveCreator::chainDisplace / chainRotate, scOOP/mc/movecreator.cpp:1075-1256):
exact running energy through the chain phase, several chain cells moving at once, and the
ensemble of the reference's own sampler with chain + single-particle moves."""
import math
import os

import numpy as np
import pytest

from test_gpu_sweep import ens, opts_text

pytestmark = pytest.mark.gpu


def test_chain_moves_keep_the_running_energy_exact():
    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.lipids_dilute(64, seed=3))
    e0 = s.all_to_all()
    st = s.simulate(nsweeps=120, seed=5, check_every=60)
    assert st.acc_chain > 0 and st.rej_chain > 0
    # N * chainprob chain attempts per sweep on average
    assert abs((st.acc_chain + st.rej_chain) / 120 - 0.2 * s.n) < 0.35 * 0.2 * s.n
    e1 = s.all_to_all()
    assert e1 != e0
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert abs(st.energy_check - e1) <= 1e-9 * max(1.0, abs(e1))
    # rigid chain moves keep every chain whole: bonded neighbours stay within a bond length
    parts = s.particles()
    pos = np.array([p.pos for p in parts]) * s.box
    d = np.linalg.norm(pos[1::3] - pos[0::3], axis=1)
    assert d.max() < 3.5
    s.close()


def test_chain_cells_move_concurrently():
    """Two bilayers of 400 lipids: the chain grid has several cells per colour."""
    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.bilayers(10, box=(12.0, 12.0, 40.0), seed=2))
    st = s.simulate(nsweeps=40, seed=7, check_every=20, chainprob=0.3)
    assert st.acc_chain > 0
    e1 = s.all_to_all()
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert abs(st.energy_check - e1) <= 1e-9 * max(1.0, abs(e1))
    s.close()


def test_chain_ensemble_matches_reference():
    from sc_gb300 import ReplicaSet, System

    g = ens("lipids_chain")
    systems = [System.from_text(opts_text(g["options"]), g["inputs"]["top.init"], g["inputs"]["config.init"])
               for _ in range(6)]
    T = g["options"]["temper"]
    R = ReplicaSet(systems, [T] * 6, ladder=list(range(6)))
    p = systems[0].default_run()
    p.check_every = 0
    E = [[] for _ in systems]
    done = 0
    # a third of the reference's sweeps (its standard error enters the combined sigma)
    nsweeps, burn = g["nsweeps"] // 3, g["burn"] // 2
    while done < nsweeps:
        _, _, en, _, _ = R.run(g["report"] * 5, exchange_every=0, seed=4243, params=p)
        done += g["report"] * 5
        if done > burn:
            for k, s in enumerate(systems):
                E[k].append(en[k] / s.n)
    R.close()
    m = np.array([np.mean(x) for x in E])
    mean, se = float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))
    ref = g["stats"]["energy_per_particle"]
    sigma = math.sqrt(se ** 2 + ref["se"] ** 2)
    assert abs(mean - ref["mean"]) <= 2.0 * sigma, (mean, se, ref)
    for s in systems:
        s.close()


def test_chain_moves_with_volume_moves_keep_the_running_energy_exact():
    """Isotropic volume moves after the chain phase: the trial energy is taken on cell
    lists built after the chains moved."""
    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.lipids_dilute(64, seed=4))
    p = s.default_run()
    p.ptype, p.volume_every, p.press, p.edge_mx = 1, 1, 0.3, 0.1
    st = s.simulate(p, nsweeps=80, seed=6, check_every=40)
    assert st.acc_chain > 0 and st.acc_vol > 0
    e1 = s.all_to_all()
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert abs(st.energy_check - e1) <= 1e-9 * max(1.0, abs(e1))
    s.close()


def test_dataflow_sweeps_give_the_colour_phase_trajectory_with_chains():
    """Single-particle and chain phases both as dataflow launches: the trajectory of the
    colour-phase launches, bit for bit."""
    from sc_gb300 import System, workloads

    texts = workloads.bilayers(10, box=(12.0, 12.0, 40.0), seed=5)
    s1, s2 = System.from_text(*texts), System.from_text(*texts)
    a = s1.simulate(nsweeps=30, seed=8, check_every=15, chainprob=0.3, variant=0)
    b = s2.simulate(nsweeps=30, seed=8, check_every=15, chainprob=0.3, variant=4)
    assert a.acc_chain > 0 and b.launches < a.launches
    assert (a.energy, a.acc_trans, a.acc_rot, a.acc_chain, a.rej_chain) == \
           (b.energy, b.acc_trans, b.acc_rot, b.acc_chain, b.rej_chain)
    assert all(list(x.pos) == list(y.pos) and list(x.dir) == list(y.dir)
               for x, y in zip(s1.particles(), s2.particles()))
    e1 = s2.all_to_all()
    assert abs(b.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    s1.close()
    s2.close()
