"""GPU move loop: bookkeeping, reproducibility and ensemble parity with the reference.

The checkerboard sampler visits configurations in another order than the
reference's sequential loop, so trajectories differ; what must agree is the
stationary distribution.  tests/golden/ens_*.json hold averages the reference's
own loop sampled (several seeds, tests/golden/make_ensemble.py); the GPU run from
the same start must match them within 2 standard errors.
"""
import json
import math
import os

import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def opts_text(extra):
    from golden.make_golden import OPTION_KEYS

    d = dict(OPTION_KEYS)
    d.update(extra)
    d["paraltemper"] = d["temper"]
    return "".join(f"{k} = {v}\n" for k, v in d.items())


def ens(name):
    with open(os.path.join(GOLDEN, f"ens_{name}.json")) as f:
        return json.load(f)


def open_ens(name):
    from sc_gb300 import System

    e = ens(name)
    s = System.from_text(opts_text(e["options"]), e["inputs"]["top.init"], e["inputs"]["config.init"])
    return e, s


def exact_energy(s):
    return s.all_to_all()


@pytest.mark.parametrize("stencil", [1, 2])
def test_running_energy_matches_exact_total(stencil):
    e, s = open_ens("psc_nvt")
    e0 = exact_energy(s)
    st = s.simulate(nsweeps=200, seed=11, check_every=50, stencil=stencil)
    assert st.moves == 200 * s.n
    assert st.acc_trans + st.rej_trans + st.acc_rot + st.rej_rot == st.moves
    assert 0.05 < (st.acc_trans + st.acc_rot) / st.moves < 0.95
    e1 = exact_energy(s)
    assert e1 != e0
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert st.max_drift <= 1e-9 * max(1.0, abs(e1))
    # the cell-list total energy of the last check equals the brute-force one
    st2 = s.simulate(nsweeps=50, seed=11, check_every=50, stencil=stencil)
    assert abs(st2.energy_check - exact_energy(s)) <= 1e-11 * max(1.0, abs(st2.energy_check))
    s.close()


def test_stencil_larger_than_shared_memory_window():
    """Cells of a long rod's cut-off holding thousands of spheres: candidates are staged
    in windows, the running energy must stay exact."""
    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.rods_in_spheres(seed=4))
    e0 = exact_energy(s)
    st = s.simulate(nsweeps=8, seed=2, check_every=4, stencil=1)
    assert st.moves == 8 * s.n and st.pairs_tested > 8 * s.n * 1100
    e1 = exact_energy(s)
    assert e1 != e0
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert abs(st.energy_check - e1) <= 1e-9 * max(1.0, abs(e1))
    s.close()


def test_same_seed_same_trajectory():
    _, s1 = open_ens("psc_nvt")
    _, s2 = open_ens("psc_nvt")
    a = s1.simulate(nsweeps=60, seed=5, check_every=0)
    b = s2.simulate(nsweeps=60, seed=5, check_every=0)
    assert a.energy == b.energy and a.acc_trans == b.acc_trans and a.acc_rot == b.acc_rot
    pa, pb = s1.particles(), s2.particles()
    assert all(list(x.pos) == list(y.pos) and list(x.dir) == list(y.dir) for x, y in zip(pa, pb))
    c = s2.simulate(nsweeps=1, seed=6, check_every=0)
    assert c.moves == s2.n
    s1.close()
    s2.close()


def test_kernel_variants_give_the_same_trajectory():
    """kColour and kColourDense are the same code under two register budgets."""
    _, s1 = open_ens("psc_nvt")
    _, s2 = open_ens("psc_nvt")
    a = s1.simulate(nsweeps=40, seed=8, check_every=0, variant=0)
    b = s2.simulate(nsweeps=40, seed=8, check_every=0, variant=1)
    assert a.energy == b.energy and a.acc_trans == b.acc_trans and a.acc_rot == b.acc_rot
    assert all(list(x.pos) == list(y.pos) for x, y in zip(s1.particles(), s2.particles()))
    s1.close()
    s2.close()


@pytest.mark.parametrize("name,stencil", [("psc_nvt", 1), ("psc_nvt", 2), ("cpsc_spa_npt", 2)])
def test_dataflow_sweep_gives_the_colour_phase_trajectory(name, stencil):
    """One dataflow launch per sweep (cells wait for their earlier-phase neighbours) moves
    every cell against the states the colour-phase launches show it: same trajectory, bit
    for bit, under both register budgets."""
    _, s1 = open_ens(name)
    _, s2 = open_ens(name)
    _, s3 = open_ens(name)
    p = s1.default_run()
    p.stencil = stencil
    a = s1.simulate(p, nsweeps=40, seed=21, check_every=20, variant=0)
    b = s2.simulate(p, nsweeps=40, seed=21, check_every=20, variant=4)
    c = s3.simulate(p, nsweeps=40, seed=21, check_every=20, variant=5)
    for x in (b, c):
        assert x.energy == a.energy and x.acc_trans == a.acc_trans and x.acc_rot == a.acc_rot
        assert x.acc_vol == a.acc_vol and x.moves == a.moves
    assert b.launches < a.launches
    for s in (s2, s3):
        assert all(list(x.pos) == list(y.pos) and list(x.dir) == list(y.dir)
                   for x, y in zip(s1.particles(), s.particles()))
    assert list(s2.box) == list(s1.box)
    for s in (s1, s2, s3):
        s.close()


@pytest.mark.parametrize("name", ["psc_nvt", "cpsc_spa_npt"])
def test_paired_passes_keep_the_running_energy_exact(name):
    """Paired passes (move m + 1 evaluated with move m, kept when move m changed nothing it
    saw): exact running energy, and both register budgets on the same trajectory."""
    _, s1 = open_ens(name)
    _, s2 = open_ens(name)
    p = s1.default_run()
    p.stencil = 1                      # larger cells: several moves per cell
    a = s1.simulate(p, nsweeps=60, seed=12, check_every=30, variant=2)
    b = s2.simulate(p, nsweeps=60, seed=12, check_every=30, variant=3)
    assert a.energy == b.energy and a.acc_trans == b.acc_trans and a.acc_rot == b.acc_rot
    assert a.moves == 60 * s1.n and a.acc_trans + a.acc_rot > 0
    e1 = s1.all_to_all()
    assert abs(a.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    assert abs(a.energy_check - e1) <= 1e-9 * max(1.0, abs(e1))
    s1.close()
    s2.close()


def test_rotations_keep_unit_vectors_and_patch_frame():
    _, s = open_ens("psc_nvt")
    s.simulate(nsweeps=100, seed=3, check_every=0)
    for p in s.particles():
        d = np.array(p.dir)
        pd = np.array(p.patchdir[0])
        assert abs(np.linalg.norm(d) - 1.0) < 1e-9
        assert abs(np.dot(d, pd)) < 1e-9
    s.close()


def test_volume_moves_change_box_and_keep_energy_exact():
    e, s = open_ens("cpsc_spa_npt")
    b0 = s.box.copy()
    p = s.default_run()
    st = s.simulate(p, nsweeps=300, seed=21, check_every=100)
    assert st.acc_vol + st.rej_vol == 300
    assert st.acc_vol > 0 and st.vol_constrained == 0
    assert not np.allclose(s.box, b0)
    e1 = exact_energy(s)
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    s.close()


@pytest.mark.parametrize("ptype", [0, 2, 3, 4, 5])
def test_pressure_couplings_change_the_box_as_the_reference(ptype):
    """MoveCreator::pressureMove (movecreator.cpp:330-546): which edges a volume move changes,
    and the running energy stays exact."""
    e, s = open_ens("cpsc_spa_npt")
    b0 = s.box.copy()
    p = s.default_run()
    st = s.simulate(p, nsweeps=200, seed=31, check_every=100, ptype=ptype)
    assert st.acc_vol + st.rej_vol == 200 and st.acc_vol > 0
    b1 = s.box
    same = np.isclose(b1, b0, rtol=0, atol=0)
    if ptype == 2:
        assert same[2] and not same[0] and np.isclose(b1[0], b1[1])
    elif ptype == 3:
        assert not same[0] and abs(np.prod(b1) / np.prod(b0) - 1) < 1e-9
    elif ptype == 4:
        assert not same[0] and same[1] and same[2]
    elif ptype == 5:
        assert same[0] and not same[1] and same[2]
    else:
        assert not same.all() and len(set(np.round(b1, 12))) > 1
    e1 = exact_energy(s)
    assert abs(st.energy - e1) <= 1e-9 * max(1.0, abs(e1))
    s.close()


def alignment_order(s):
    """Updater::alignmentOrder (scOOP/mc/updater.cpp:466-481)."""
    parts = s.particles()
    box = s.box
    pos = np.array([p.pos for p in parts])
    d = np.array([p.dir for p in parts])
    r = pos[:, None, :] - pos[None, :, :]
    r = (r - np.round(r)) * box
    close = (r * r).sum(-1) < 1.5 * 1.5
    iu = np.triu_indices(len(parts), 1)
    return float((d @ d.T)[iu][close[iu]].sum())


def sample(systems, golden, nsweeps, seed):
    """Independent trajectories (one per system, same start, own Philox stream) moved
    together as a replica batch without exchanges; returns per-trajectory series."""
    from sc_gb300 import ReplicaSet

    T = golden["options"]["temper"]
    R = ReplicaSet(systems, [T] * len(systems), ladder=list(range(len(systems))))
    p = systems[0].default_run()
    p.check_every = 0
    rep = golden["report"]
    E = [[] for _ in systems]
    A = [[] for _ in systems]
    V = [[] for _ in systems]
    done = 0
    while done < nsweeps:
        st, _, en, _, _ = R.run(rep, exchange_every=0, seed=seed, params=p)
        done += rep
        if done > golden["burn"]:
            for k, s in enumerate(systems):
                E[k].append(en[k] / s.n)
                A[k].append(alignment_order(s) / s.n)
                V[k].append(float(np.prod(s.box)) / s.n)
    R.close()
    return [np.array(x) for x in E], [np.array(x) for x in A], [np.array(x) for x in V]


def mean_se(series):
    """Mean and standard error from the means of independent trajectories."""
    m = np.array([x.mean() for x in series])
    return float(m.mean()), float(m.std(ddof=1) / math.sqrt(len(m)))


@pytest.mark.parametrize("name", ["psc_nvt", "cpsc_spa_npt"])
def test_ensemble_matches_reference(name):
    from sc_gb300 import System

    g = ens(name)
    systems = [System.from_text(opts_text(g["options"]), g["inputs"]["top.init"], g["inputs"]["config.init"])
               for _ in range(6)]
    E, A, V = sample(systems, g, g["nsweeps"], seed=4242)
    checks = [("energy_per_particle", E), ("alignment_per_particle", A)]
    if g["options"].get("ptype") == 1:
        checks.append(("volume_per_particle", V))
    report = {}
    for key, x in checks:
        m, se = mean_se(x)
        ref = g["stats"][key]
        sigma = math.sqrt(se ** 2 + ref["se"] ** 2)
        report[key] = (m, se, ref["mean"], ref["se"])
        assert abs(m - ref["mean"]) <= 2.0 * sigma, report
    for s in systems:
        s.close()


def test_dataflow_wait_limit_reports_and_recovers():
    """The dataflow sweep's bounded wait: with a limit of one poll, a cell that finds an
    earlier-phase neighbour unfinished gives up, the kernel returns and the call reports
    SC_ERR_DEVICE; the context stays usable, and the next run (default limit) recomputes the
    exact energy and keeps it exact."""
    from sc_gb300 import ScError, System

    g = goldens.load("syn_cpsc_spa_npt_small")
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    s.simulate(nsweeps=2, seed=5, variant=4, check_every=0)
    failed = 0
    for k in range(5):
        try:
            s.simulate(nsweeps=4, seed=6 + k, variant=4, check_every=0, flow_wait_polls=1)
        except ScError as ex:
            assert "DEVICE" in str(ex) and "waited too long" in str(ex), str(ex)
            failed += 1
    assert failed > 0
    st = s.simulate(nsweeps=5, seed=20, variant=4, check_every=0)
    assert st.sweeps == 5
    exact = s.all_to_all()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
    s.close()


def test_tuner_restores_state_and_is_used():
    """sc_tune times every candidate launch shape on the current state and leaves that state
    as it found it; runs with variant = -1 then use its choice, and stay exact."""
    from sc_gb300 import System

    g = goldens.load("syn_cpsc_spa_npt_small")
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    s.simulate(nsweeps=3, seed=2, check_every=0)
    before = s.particles()
    box = s.box.copy()
    p = s.default_run()
    p.seed, p.check_every = 4, 0
    best, rates = s.tune(p, sweeps=2)
    variants = [0, 1, 2, 3, 4, 5, 8, 9]
    assert len(rates) == 3 * len(variants) and max(rates) > 0
    assert best.stencil in (1, 2, 3) and best.variant in variants
    assert rates[(best.stencil - 1) * len(variants) + variants.index(best.variant)] == max(rates)
    after = s.particles()
    assert np.array_equal(s.box, box)
    for k in range(s.n):
        assert list(after[k].pos) == list(before[k].pos) and list(after[k].dir) == list(before[k].dir)
    st = s.simulate(p, nsweeps=4, variant=-1)
    exact = s.all_to_all()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact))
    s.close()


def _texts(name):
    """Seeded starts without overlaps (the golden fixtures start with overlap energies up to
    1e17, which a running energy cannot carry to 1e-9 of the relaxed total in FP64)."""
    from sc_gb300 import workloads

    if name == "lipids":            # three-bead lipids with bonds and chain moves
        return workloads.lipids_dilute(64, seed=3)
    if name == "mixture":           # CPSC + SPA, NPT with isotropic volume moves
        return workloads.npt_cpsc_spa(300, seed=2)
    if name == "psc":
        return workloads.nvt_psc(250, phi=0.15, seed=2)
    inp = goldens.load(name)["inputs"]
    return inp["options"], inp["top.init"], inp["config.init"]


@pytest.mark.parametrize("variant", [8, 9])
@pytest.mark.parametrize("name", ["mixture", "lipids", "psc"])
def test_warp_cells_exact_and_reproducible(name, variant):
    """The warp-per-cell dataflow sweep (variant bit 3): the running energy stays the exact
    total through moves, volume moves and chain moves, and a rerun from the same start with
    the same seed reproduces the state bit for bit."""
    from sc_gb300 import System

    runs = []
    for _ in range(2):
        s = System.from_text(*_texts(name))
        st = s.simulate(nsweeps=30, seed=17, variant=variant, check_every=10)
        exact = s.all_to_all()
        assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
        assert st.max_drift <= 1e-9 * max(1.0, abs(exact))
        assert st.acc_trans + st.acc_rot > 0 and st.moves >= 30 * s.n
        runs.append((st.energy, [tuple(q.pos) + tuple(q.dir) for q in s.particles()], tuple(s.box)))
        s.close()
    assert runs[0] == runs[1]


@pytest.mark.parametrize("name", ["syn_cpsc_spa_npt_small", "syn_psc_nvt_small", "syn_bilayer_small", "lipids",
                                  "mixture"])
def test_warp_cells_follow_the_cta_kernel(name):
    """Same proposals, screens and pair energies as the CTA-per-cell dataflow kernel: from the
    same start and seed both take the same decisions (the same states), and their running
    energies differ only by the summation order."""
    from sc_gb300 import System

    out = {}
    for v in (4, 8):
        s = System.from_text(*_texts(name))
        st = s.simulate(nsweeps=6, seed=23, variant=v, stencil=2, check_every=0)
        out[v] = (st, [tuple(q.pos) + tuple(q.dir) for q in s.particles()], tuple(s.box))
        s.close()
    a, b = out[4], out[8]
    assert (a[0].acc_trans, a[0].acc_rot, a[0].acc_vol) == (b[0].acc_trans, b[0].acc_rot, b[0].acc_vol)
    assert a[1] == b[1] and a[2] == b[2]
    assert a[0].pairs_tested == b[0].pairs_tested
    if not name.startswith("syn_"):
        # the golden starts hold overlap energies up to 1e16, whose rounding the two summation
        # orders carry differently; on clean starts the running energies agree closely
        assert abs(a[0].energy - b[0].energy) <= 1e-11 * max(1.0, abs(a[0].energy))


def test_axial_rotations_turn_about_the_particle_axis():
    """options coneAngle > 0 (MoveCreator::partAxialRotate): rotation axes lie in a cone of that
    angle around the particle's own axis.  With a cone of 1e-4 degrees the axes barely move
    while the patches turn freely, and the running energy stays exact."""
    from sc_gb300 import System, workloads

    opts, top, cfg = workloads.nvt_psc(200, phi=0.1, seed=9)
    opts = opts.replace("transmx = 0.4", "transmx = 0.05") + "coneAngle = 0.0001\n"
    s = System.from_text(opts, top, cfg)
    before = s.particles()
    st = s.simulate(nsweeps=20, seed=5, check_every=0)
    after = s.particles()
    dd = max(max(abs(a.dir[k] - b.dir[k]) for k in range(3)) for a, b in zip(after, before))
    dp = max(max(abs(a.patchdir[0][k] - b.patchdir[0][k]) for k in range(3)) for a, b in zip(after, before))
    assert st.acc_rot > 100
    assert dd < 1e-4, dd
    assert dp > 0.1, dp
    exact = s.all_to_all()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact))
    s.close()
