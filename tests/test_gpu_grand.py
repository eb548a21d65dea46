"""Grand-canonical insert / delete moves on the GPU (MoveCreator::muVTMove,
scOOP/mc/movecreator.cpp:797-924, one move every nGrandCanon sweeps, updater.cpp:164-179).

Ensemble parity: tests/golden/ens_gc_spa.json and ens_gc_psc.json hold the mean particle
count (from the reference's movie frames) and the mean total energy (energy.dat) sampled
by the reference's own loop (oracle/_ref/sc_ref, tests/golden/make_ensemble.py) for
attractive spheres exchanged with a reservoir (32 seeds), and for patchy spherocylinders
exchanged among fixed spheres (48 seeds; the species listed last, so removals inside its
block shift the particles behind).  The GPU runs trajectories from the same start for the
same sweeps (the spheres eight, one at a time; the spherocylinders as many as the
reference, as one batch); both means must agree within 2 combined standard errors.

Exactness: the running energy (the moves' energy changes, insertions and removals
included) equals the exact total energy after the run; the particle vector keeps the
reference's order (each molecule type in its block, the inserted particles of a species at
its block's end); capacity growth from an empty box; chains before the species with chain
moves; the schedule over calls (sweep_offset); bitwise reproducibility; replica exchange
with the grand-canonical term.
"""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case(name):
    with open(os.path.join(GOLDEN, f"ens_{name}.json")) as f:
        g = json.load(f)
    from golden.make_golden import OPTION_KEYS

    o = dict(OPTION_KEYS)
    o.update(g["options"])
    o["paraltemper"] = o["temper"]
    return g, "".join(f"{k} = {v}\n" for k, v in o.items()), g["inputs"]["top.init"], g["inputs"]["config.init"]


def _check_layout(s):
    """Each molecule type in one block in [Molecules] order; the species counts match."""
    mt = np.array([p.molType for p in s.particles()], dtype=np.int64)
    assert np.all(np.diff(mt) >= 0)
    for g in s.grand_stats():
        assert int(np.sum(mt == g.mol_type)) == g.count


@pytest.mark.parametrize("name,batched", [("gc_spa", False), ("gc_psc", True)])
def test_ensemble_matches_reference(name, batched):
    """gc_spa: one system at a time through sc_simulate; gc_psc: the trajectories moved
    together as a replica batch without exchanges (each keeps its own slots and count)."""
    from sc_gb300 import ReplicaSet, System

    g, opts, top, cfg = _case(name)
    rep, burn, nsw = g["report"], g["burn"], g["nsweeps"]
    N, E = [], []
    groups = [list(range(g["seeds"]))] if batched else [[k] for k in range(min(8, g["seeds"]))]
    for group in groups:
        systems = [System.from_text(opts, top, cfg) for _ in group]
        p = systems[0].default_run()
        p.check_every = 0
        p.seed = 7000 + group[0]
        R = ReplicaSet(systems, [float(g["options"]["temper"])] * len(systems),
                       ladder=list(range(len(systems)))) if batched else None
        n_ser = [[] for _ in group]
        e_ser = [[] for _ in group]
        done = 0
        while done < nsw:
            if batched:
                _, _, en, _, _ = R.run(rep, exchange_every=0, seed=p.seed, params=p, sweep_offset=done)
            else:
                en = [systems[0].simulate(p, nsweeps=rep, sweep_offset=done).energy]
            done += rep
            if done > burn:
                for k, s in enumerate(systems):
                    n_ser[k].append(s.n)
                    e_ser[k].append(en[k])
        if R is not None:
            R.close()
        for k, s in enumerate(systems):
            exact = s.all_to_all()
            st = s.simulate(p, nsweeps=0)
            assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
            assert st.particles == s.n
            _check_layout(s)
            N.append(np.array(n_ser[k], dtype=float))
            E.append(np.array(e_ser[k]))
            s.close()
    report = {}
    for key, ser in (("particles", N), ("energy_total", E)):
        m = np.array([x.mean() for x in ser])
        mean, se = float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))
        ref = g["stats"][key]
        report[key] = (mean, se, ref["mean"], ref["se"])
    print(f"grand-canonical ensemble {name} (GPU mean, se, reference mean, se):", report)
    for key, (mean, se, rm, rse) in report.items():
        assert abs(mean - rm) <= 2.0 * math.sqrt(se ** 2 + rse ** 2), report


def test_batched_systems_reproduce_single_runs():
    """Grand-canonical systems moved together as a replica batch (no exchanges) follow the
    same trajectories, bit for bit, as the same systems run one at a time with the seeds the
    batch derives for them: the moves, the counts and the particle order do not depend on
    the batch."""
    from test_gpu_replicas import GOLDEN
    from sc_gb300 import ReplicaSet, System

    g, opts, top, cfg = _case("gc_psc")
    sysA = [System.from_text(opts, top, cfg) for _ in range(3)]
    sysB = [System.from_text(opts, top, cfg) for _ in range(3)]
    R = ReplicaSet(sysA, [1.0] * 3, ladder=[0, 1, 2])
    p = sysA[0].default_run()
    p.check_every = 0
    _, _, E, _, _ = R.run(200, exchange_every=0, seed=77, params=p, stencil=2)
    R.close()
    for k, s in enumerate(sysB):
        q = s.default_run()
        q.check_every = 0
        single = s.simulate(q, nsweeps=200, seed=(77 + GOLDEN * (k + 1)) % (1 << 64), stencil=2)
        assert sysA[k].n == s.n, (k, sysA[k].n, s.n)
        pa, pb = sysA[k].particles(), s.particles()
        assert [list(x.pos) for x in pa] == [list(y.pos) for y in pb]
        assert single.energy == E[k]
    for s in sysA + sysB:
        s.close()


def test_energy_checks_during_grand_and_chain_moves():
    """The exact-energy checks inside a run (check_every) see the particles where they are:
    after grand-canonical moves (slots moved) and chain moves (particles left their cells) the
    cell list is built anew, so the largest drift stays at rounding level."""
    from sc_gb300 import System, workloads

    opts_text, top, config = workloads.lipids_dilute(24, seed=5)
    top = top.replace("[System]", "S: {\nparticles: 9\nACTIVITY: 0.05\n}\n[System]", 1)
    top = top.replace("[Molecules]", "S 9 SPA 0.5 1.0 1.1225 0.3775\n[Molecules]", 1)
    top = top.rstrip("\n") + "\nS 0\n"
    o = dict(l.split(" = ") for l in opts_text.strip().splitlines())
    o.update(nGrandCanon="1", chainprob="0.2")
    s = System.from_text("".join(f"{k} = {v}\n" for k, v in o.items()), top, config)
    p = s.default_run()
    p.check_every = 7
    p.seed = 4
    st = s.simulate(p, nsweeps=300)
    assert st.acc_insert > 0 and st.acc_chain > 0
    assert st.max_drift <= 1e-9 * max(1.0, abs(st.energy)), (st.max_drift, st.energy)
    s.close()


def test_growth_from_an_empty_box():
    """A crowding species from an empty box: the free slots run out and grow (first 256),
    the count passes them, and the running energy stays exact."""
    from golden.make_golden import options_text, top_text
    from sc_gb300 import System

    top = top_text([("A", 1, "SPA", [1.0, 1.0, 1.1225, 0.5])], [("A", [1], ["ACTIVITY: 50.0"])], [("A", 0)])
    s = System.from_text(options_text(nGrandCanon=1, transmx=0.4, temper=1.0), top, "9 9 9\n")
    p = s.default_run()
    p.check_every = 0
    p.seed = 11
    total = 0
    for _ in range(8):
        st = s.simulate(p, nsweeps=250, sweep_offset=total)
        total += 250
        exact = s.all_to_all()
        assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
    assert s.n > 300, s.n
    (g,) = s.grand_stats()
    assert g.steps == 2000 and g.ins_acc - g.del_acc == s.n
    assert g.ins_acc + g.ins_rej + g.del_acc + g.del_rej == g.steps
    pos = np.array([p.pos for p in s.particles()])
    assert np.all(np.isfinite(pos))
    s.close()


def test_chains_before_the_species():
    """Three-bead lipids with chain moves, then solvent spheres exchanged with a reservoir:
    the chains keep their slots, the chain phase follows the count, the energy stays exact."""
    from sc_gb300 import System, workloads

    opts_text, top, config = workloads.lipids_dilute(24, seed=5)
    top = top.replace("[System]", "S: {\nparticles: 9\nACTIVITY: 0.05\n}\n[System]", 1)
    top = top.replace("[Molecules]", "S 9 SPA 0.5 1.0 1.1225 0.3775\n[Molecules]", 1)
    top = top.rstrip("\n") + "\nS 0\n"
    o = dict(l.split(" = ") for l in opts_text.strip().splitlines())
    o.update(nGrandCanon="2", chainprob="0.2")
    s = System.from_text("".join(f"{k} = {v}\n" for k, v in o.items()), top, config)
    p = s.default_run()
    p.check_every = 0
    p.seed = 3
    st = s.simulate(p, nsweeps=400)
    exact = s.all_to_all()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
    assert st.acc_chain > 0 and st.acc_insert > 0
    mt = np.array([q.molType for q in s.particles()])
    assert np.all(mt[:72] == 0) and np.all(mt[72:] == 1) and s.n == 72 + s.grand_stats()[0].count
    s.close()


def test_schedule_counts_from_the_loop_start():
    from sc_gb300 import System

    g, opts, top, cfg = _case("gc_spa")
    s = System.from_text(opts.replace("nGrandCanon = 1", "nGrandCanon = 3"), top, cfg)
    p = s.default_run()
    p.check_every = 0
    s.simulate(p, nsweeps=10, sweep_offset=0)       # sweeps 1..10: moves after 3, 6, 9
    assert s.grand_stats()[0].steps == 3
    s.simulate(p, nsweeps=10, sweep_offset=11)      # sweeps 12..21: after 12, 15, 18, 21
    assert s.grand_stats()[0].steps == 7
    s.close()


def test_bitwise_reproducible():
    from sc_gb300 import System

    g, opts, top, cfg = _case("gc_psc")
    out = []
    for _ in range(2):
        s = System.from_text(opts, top, cfg)
        p = s.default_run()
        p.seed = 99
        st = s.simulate(p, nsweeps=300)
        out.append((st.energy, s.n, np.array([q.pos for q in s.particles()]).tobytes()))
        s.close()
    assert out[0] == out[1]


def test_replica_exchange_with_grand_moves():
    """Grand-canonical replicas: every exchange decision is the reference's rule with its
    grand-canonical term (movecreator.cpp:713-745: change = (1/T_i - 1/T_j)(E_i - E_j) +
    (1/T_i - 1/T_j) chemPot T_i (N_i - N_j), NVT), restated on the energies, counts,
    temperatures and the uniforms of the exchange's own stream; each call makes a
    grand-canonical move after its first sweep (grand_every 2 from loop sweep 2) and the
    exchange after its second, so the call's final energies and counts are the ones the
    exchange saw.  Running energies stay exact and the counts follow the device."""
    from test_gpu_replicas import _M, _uniforms
    from sc_gb300 import ReplicaSet, System

    g, opts, top, cfg = _case("gc_spa")
    systems = [System.from_text(opts, top, cfg) for _ in range(4)]
    chem = systems[0].grand_stats()[0].chem_pot
    temps = list(np.geomspace(0.9, 1.0, 4))
    R = ReplicaSet(systems, temps, ladder=[0] * 4)
    p = systems[0].default_run()
    p.grand_every, p.sweep_offset, p.check_every = 2, 1, 0
    seed = 31
    u_seed = seed ^ 0xA5A5A5A5
    T = np.array(temps)
    decided = accepted = 0
    counts = set()
    for ev in range(40):
        st, T_after, E, tried, acc = R.run(2, exchange_every=2, seed=seed, params=p)
        N = np.array([s.n for s in systems], dtype=float)
        counts.update(N.tolist())
        ladder = list(np.argsort(T, kind="stable"))
        want = T.copy()
        u = _uniforms(u_seed, 0xFFFFFFE0, ev & _M, ev >> 32)
        for k in range(ev & 1, len(ladder) - 1, 2):
            ri, rj = ladder[k], ladder[k + 1]
            change = (1.0 / T[ri] - 1.0 / T[rj]) * (E[ri] - E[rj])
            change += (1.0 / T[ri] - 1.0 / T[rj]) * chem * T[ri] * (N[ri] - N[rj])
            x = next(u)
            if change >= 0.0 or math.exp(change) > x:
                want[ri], want[rj] = T[rj], T[ri]
                accepted += 1
            decided += 1
        assert np.array_equal(T_after, want), (ev, T, T_after, want, E, N)
        T = T_after
    assert 0 < accepted < decided and len(counts) > 1
    R.close()
    for s in systems:
        exact = s.all_to_all()
        st = s.simulate(p, nsweeps=0)
        assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact))
        _check_layout(s)
        s.close()


def test_output_loop_writes_top_last(tmp_path):
    from sc_gb300 import System, updater

    g, opts, top, cfg = _case("gc_spa")
    s = System.from_text(opts, top, cfg)
    tot = updater.run(s, 200, report=50, movie=50, directory=str(tmp_path))
    text = (tmp_path / "top.last").read_text()
    assert text.endswith(f"[System]\nA {s.n}\n")
    counts = [int(l.split()[0]) for l in (tmp_path / "movie").read_text().splitlines() if len(l.split()) == 1]
    assert len(counts) == 4 and counts[-1] == s.n
    assert tot["grand"][0]["steps"] == 200
    s.close()
