"""Wang-Landau on the GPU move loop.

WangLandau (scOOP/mc/wanglandau.h, wanglandau.cpp) biases each move by the weights of
the order parameters and lowers the visited bin's weight by alpha after every move.  On
the GPU the cells holding the order parameters' particles move after the sweep's other
cells (kWlCells), so each of their moves sees the current bins and weights; every other
move visits the current bin.  Checked here:

* adaptive weights of the xy distance of two particles converge to the reference's own
  runs of the same system (tests/golden/wl/cases.json.gz, three seeds of the reference's
  main) and to -T ln d, the density of states of the projected distance;
* fixed weights w(o) of particle 0's axis z component give a histogram ln H = w / T + c
  (the orientation is uniform without the bias): the bias enters with the reference's sign;
* the histogram counts every move, volume moves included; the current bins follow the
  state (box lengths, distances, orientation, contact count); the running energy stays
  exact; runs are reproducible and the dataflow sweep gives the colour-phase launches'
  trajectory;
* fixed weights linear in the number of spheres in contact with particle 0 (order 7), with
  and without volume moves, sample the reference's own distribution of the count.
"""
import gzip
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    with gzip.open(os.path.join(HERE, "golden", "wl", "cases.json.gz"), "rt") as f:
        return {c["name"]: c for c in json.load(f)["cases"]}


CASES = cases()


def open_case(name):
    from sc_gb300 import System

    c = CASES[name]
    inp = c["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    s.wl_load(text=inp["wl.dat"])
    return s, c


def test_adaptive_distance_weights_match_reference_and_density_of_states():
    # The reference's walker reached alpha ~ 3e-5 in 60,000 sweeps; here displacements that
    # leave their cell are rejected, so the walker diffuses more slowly and reaches alpha
    # ~ 5e-4 (ten halvings): its weights carry more noise, hence the tolerances.
    s, c = open_case("o4_pair")
    p = s.default_run()
    p.variant = 4
    st = s.simulate(p, nsweeps=60000, seed=5)
    i = s.wl_info()
    w, h = s.wl_weights()
    s.close()
    assert st.sweeps == 60000
    assert i.updates >= 7, (i.updates, i.alpha)          # the histogram went flat again and again
    lo, hi = 2, 29                                        # d in (0.2, 2.9]: below L/2, well sampled
    ref = np.array([r["weights"] for r in c["ref_runs"]])[:, lo:hi]
    ref = (ref - ref.mean(1, keepdims=True)).mean(0)
    got = w[lo:hi] - w[lo:hi].mean()
    rms = float(np.sqrt(((got - ref) ** 2).mean()))
    assert rms < 0.45, (rms, np.round(got, 2), np.round(ref, 2))
    centre = 0.05 + 0.1 * np.arange(len(w))
    sel = (centre > 1.4) & (centre < 2.9)
    slope = np.polyfit(np.log(centre[sel]), w[sel], 1)[0]
    assert -2.0 < slope < -0.6, slope                     # w = -T ln d + c, T = 1


def test_weights_wall_keeps_the_distance_inside_a_window():
    # fixed weights 0 inside bins 20..30 and -1e4 outside: exp(-1e4) is 0 in double, so a
    # move out of the window is never accepted (a sign error would pin the walker outside)
    s, c = open_case("o4_pair")
    lines = c["inputs"]["wl.dat"].splitlines()
    out = ["0.0"]
    for k, line in enumerate(lines[1:]):
        o = line.split()[0]
        out.append(f"{o} {0.0 if 20 <= k <= 30 else -1e4} 0")
    s.wl_load(text="\n".join(out) + "\n")
    assert 20 <= s.wl_info().currorder[0] <= 30
    p = s.default_run()
    p.variant = 4
    s.simulate(p, nsweeps=4000, seed=17)
    _, h = s.wl_weights()
    s.close()
    assert h[:20].sum() == 0 and h[31:].sum() == 0
    assert (h[21:30] > 0).all()


def test_fixed_weights_bias_the_orientation_with_the_reference_sign():
    s, c = open_case("o3_orient")
    i0 = s.wl_info()
    assert i0.alpha == 0.0                                # 1e-12 in the file: fixed weights
    w0, h0 = s.wl_weights()
    p = s.default_run()
    st = s.simulate(p, nsweeps=50000, seed=9)
    w1, h1 = s.wl_weights()
    s.close()
    assert np.array_equal(w0, w1)                         # alpha = 0: the weights stay
    H = (h1 - h0).astype(float)
    o = -1.0 + 0.05 * np.arange(len(H))
    sel = H[:40] > 0
    assert sel.sum() >= 38
    slope, _ = np.polyfit(o[:40][sel], np.log(H[:40][sel]), 1, w=np.sqrt(H[:40][sel]))
    assert abs(slope - 1.5) < 0.15, slope                 # ln H = w / T + c with w = 1.5 o, T = 1
    assert st.acc_rot > 10000


def _contacts(parts, box, wlmtype):
    # WangLandau::contParticlesAll (wanglandau.h:603-615, WL_CONTACTS = 36)
    p0 = np.array(parts[0].pos)
    n = 0
    for q in parts[1:]:
        if q.type != wlmtype:
            continue
        d = np.array(q.pos) - p0
        r = np.array(box) * (d - np.rint(d))
        n += float(r @ r) < 36.0
    return n


@pytest.mark.parametrize("name", ["o8_o9", "o1_bath", "o1_o3", "o4_pair", "o7_contact", "o7_npt"])
def test_histogram_counts_every_move_and_bins_follow_the_state(name):
    s, c = open_case(name)
    _, h0 = s.wl_weights()
    p = s.default_run()
    p.check_every = 100
    st = s.simulate(p, nsweeps=400, seed=3)               # below the first flatness check
    i = s.wl_info()
    _, h1 = s.wl_weights()
    parts = s.particles()
    box = s.box
    s.close()
    moves = st.moves + st.acc_vol + st.rej_vol
    assert int((h1 - h0).sum()) == moves
    assert st.moves == 400 * c["n"]
    assert st.max_drift <= 1e-9 * max(1.0, abs(st.energy)), (st.max_drift, st.energy)
    for k in range(i.dim):
        m, lo, d = i.wlm[k], i.minorder[k], i.dorder[k]
        if m == 8:
            want = math.ceil((box[0] - lo) / d)
        elif m == 9:
            want = math.ceil((box[1] - lo) / d)
        elif m == 3:
            want = math.floor((parts[0].dir[2] - lo) / d)
        elif m == 4:
            dx, dy = parts[0].pos[0] - parts[1].pos[0], parts[0].pos[1] - parts[1].pos[1]
            rx, ry = box[0] * (dx - np.rint(dx)), box[1] * (dy - np.rint(dy))
            want = math.ceil((math.sqrt(rx * rx + ry * ry) - lo) / d)
        elif m == 7:
            want = math.ceil((_contacts(parts, box, 2) - lo) / d)
        else:               # 1: z of particle 0 relative to the centre the device tracks
            want = math.ceil(((parts[0].pos[2] - i.syscm[2]) * box[2] - lo) / d)
        assert i.currorder[k] == want, (name, k, i.currorder[k], want)
    if name in ("o8_o9", "o7_npt"):
        assert st.acc_vol > 0


@pytest.mark.parametrize("name", ["o1_o3", "o4_pair", "o7_contact"])
def test_runs_are_reproducible_and_dataflow_matches_phase_launches(name):
    out = []
    for variant in (0, 0, 4):
        s, c = open_case(name)
        p = s.default_run()
        p.variant = variant
        st = s.simulate(p, nsweeps=300, seed=21)
        w, h = s.wl_weights()
        pos = np.array([list(q.pos) for q in s.particles()])
        out.append((w, h, pos, st.energy))
        s.close()
    for w, h, pos, e in out[1:]:
        assert np.array_equal(w, out[0][0])
        assert np.array_equal(h, out[0][1])
        assert np.array_equal(pos, out[0][2])
        assert e == out[0][3]


@pytest.mark.parametrize("variant", [0, 4])
def test_chain_moves_visit_the_current_bin(variant):
    # a CPSC particle above a small lipid bilayer (chain moves on), orders 1 and 3
    from sc_gb300 import System, workloads

    opts, top, cfg, wl = workloads.protein_bilayer(n_side=8, box=(26.0, 26.0, 30.0), seed=2)
    s = System.from_text(opts, top, cfg)
    s.wl_load(text=wl)
    _, h0 = s.wl_weights()
    p = s.default_run()
    p.variant = variant
    p.check_every = 50
    st = s.simulate(p, nsweeps=300, seed=8)
    i = s.wl_info()
    _, h1 = s.wl_weights()
    parts = s.particles()
    box = s.box
    s.close()
    chain = st.acc_chain + st.rej_chain
    assert chain > 0
    assert int((h1 - h0).sum()) == st.moves + chain
    assert st.max_drift <= 1e-9 * max(1.0, abs(st.energy)), (st.max_drift, st.energy)
    assert i.currorder[1] == math.floor((parts[0].dir[2] - i.minorder[1]) / i.dorder[1])
    assert i.currorder[0] == math.ceil(((parts[0].pos[2] - i.syscm[2]) * box[2] - i.minorder[0]) / i.dorder[0])


def test_reference_membrane_test_runs_with_its_converged_weights():
    """The reference's own Wang-Landau test (Tests/SC_PSC_MEMBRANE_WANG: a CPSC protein of
    length 6 above 200 three-bead lipids in a 10.9 x 10.9 x 50 box, orders 1 and 3, volume
    moves at constant z (ptype 2), chain moves) with the converged weights of its legacy run.
    The protein makes the cutoff about 9, so the grid is one cell wide in x and y and the
    bilayer's 600 particles share a cell (more than a cell stages in shared memory: read from
    the cell list).  Every move, volume move and chain move visits the histogram once, the
    bins follow the state, the running energy stays exact."""
    s, c = open_case("membrane_ref")
    _, h0 = s.wl_weights()
    p = s.default_run()
    assert p.ptype == 2 and p.volume_every == 1 and p.chainprob == 0.1
    p.check_every = 50
    st = s.simulate(p, nsweeps=200, seed=5)
    i = s.wl_info()
    _, h1 = s.wl_weights()
    parts = s.particles()
    box = s.box
    exact = s.all_to_all()            # over all pairs, no cell list
    s.close()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (st.energy, exact)
    chain = st.acc_chain + st.rej_chain
    assert chain > 0 and st.moves == 200 * c["n"] and st.acc_vol + st.rej_vol == 200
    assert st.acc_trans > 0 and st.acc_rot > 0
    assert int((h1 - h0).sum()) == st.moves + chain + st.acc_vol + st.rej_vol
    assert st.max_drift <= 1e-9 * max(1.0, abs(st.energy)), (st.max_drift, st.energy)
    assert i.currorder[1] == math.floor((parts[0].dir[2] - i.minorder[1]) / i.dorder[1])
    assert i.currorder[0] == math.ceil(((parts[0].pos[2] - i.syscm[2]) * box[2] - i.minorder[0]) / i.dorder[0])


def test_order1_fixed_weights_sample_the_reference_distribution():
    """Order 1 under fixed weights (a harmonic well in the height of particle 0 above the
    system centre, alpha 0) in an interacting bath: the mean and the variance of the visited
    bin over six trajectories agree with six runs of the reference's own loop within 2
    combined standard errors.  This bounds the effect of the stated deviation -- the centre's
    shifts by the other cells' displacements are not biased (they are in the reference)."""
    from sc_gb300 import ReplicaSet, System

    c = CASES["o1_fixed"]
    inp = c["inputs"]
    ws = []
    for _ in c["ref_runs"]:
        s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
        s.wl_load(text=inp["wl.dat"])
        ws.append(s)
    h0 = [s.wl_weights()[1] for s in ws]
    R = ReplicaSet(ws, temperatures=[1.0] * len(ws), ladder=list(range(len(ws))))
    R.run(20000, exchange_every=0, seed=31, variant=4)
    R.close()

    def moments(h):
        h = np.asarray(h, dtype=float)
        i = np.arange(len(h))
        m = (h * i).sum() / h.sum()
        return m, (h * (i - m) ** 2).sum() / h.sum()

    got = np.array([moments(s.wl_weights()[1] - h) for s, h in zip(ws, h0)])
    ref = np.array([moments(r["hist"]) for r in c["ref_runs"]])
    w0 = ws[0].wl_weights()[0]
    for s in ws:
        assert np.array_equal(s.wl_weights()[0], w0)                       # alpha 0: fixed
    for s in ws:
        s.close()
    print("order 1 fixed weights (GPU, reference: mean bin, bin variance):", got.mean(0), ref.mean(0))
    for k, name in enumerate(("mean bin", "bin variance")):
        se = math.sqrt(got[:, k].var(ddof=1) / len(got) + ref[:, k].var(ddof=1) / len(ref))
        assert abs(got[:, k].mean() - ref[:, k].mean()) <= 2.0 * se, (name, got[:, k], ref[:, k])


@pytest.mark.parametrize("name", ["o7_contact", "o7_npt"])
def test_contact_order_fixed_weights_sample_the_reference_distribution(name):
    """Order 7 under fixed weights 0.08 per sphere in contact with particle 0 (alpha 0), in
    an interacting bath, without and with isotropic volume moves (which recount the contacts
    in the trial box): as many walkers as the reference ran (a batch, each with its own
    table), the mean and the spread of the visited bin agree with the reference's own runs
    (3 combined standard errors; spreads within 25 %), and each walker's bin is the count
    recomputed from its final state."""
    from sc_gb300 import ReplicaSet, System

    c = CASES[name]
    inp = c["inputs"]
    nsweeps = int(next(l for l in inp["options"].splitlines() if l.split("=")[0].strip() == "nsweeps").split("=")[1])
    ws = []
    for _ in c["ref_runs"]:
        s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
        s.wl_load(text=inp["wl.dat"])
        ws.append(s)
    h0 = [s.wl_weights()[1] for s in ws]
    w0 = ws[0].wl_weights()[0]
    R = ReplicaSet(ws, temperatures=[1.0] * len(ws), ladder=list(range(len(ws))))
    R.run(nsweeps, exchange_every=0, seed=41, variant=4)
    R.close()

    def moments(h):
        h = np.asarray(h, dtype=float)
        i = np.arange(len(h))
        m = (h * i).sum() / h.sum()
        return m, math.sqrt((h * (i - m) ** 2).sum() / h.sum())

    got = np.array([moments(s.wl_weights()[1] - h) for s, h in zip(ws, h0)])
    ref = np.array([moments(r["hist"]) for r in c["ref_runs"]])
    for s in ws:
        assert np.array_equal(s.wl_weights()[0], w0)                       # alpha 0: fixed
        i = s.wl_info()
        want = math.ceil((_contacts(s.particles(), s.box, 2) - i.minorder[0]) / i.dorder[0])
        assert i.currorder[0] == want
        s.close()
    print(f"order 7 fixed weights {name} (GPU, reference: mean bin, spread):", got.mean(0), ref.mean(0))
    se = math.sqrt(got[:, 0].var(ddof=1) / len(got) + ref[:, 0].var(ddof=1) / len(ref))
    assert abs(got[:, 0].mean() - ref[:, 0].mean()) <= 3.0 * se, (got[:, 0], ref[:, 0])
    assert abs(got[:, 1].mean() - ref[:, 1].mean()) <= 0.25 * ref[:, 1].mean(), (got[:, 1], ref[:, 1])


def test_walkers_share_one_table():
    # four walkers of the two-particle distance case update one table (the reference's
    # multiple walkers): every walker's moves count in the shared histogram, the owner's
    # flatness checks halve the shared alpha, and the weights approach the reference's
    from sc_gb300 import ReplicaSet, System

    c = CASES["o4_pair"]
    inp = c["inputs"]
    ws = []
    for k in range(4):
        s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
        s.wl_load(text=inp["wl.dat"])
        ws.append(s)
    System.wl_share(ws)
    R = ReplicaSet(ws, temperatures=[1.0] * 4)
    st, _, _, _, _ = R.run(400, exchange_every=0, seed=4, variant=4)
    _, h = ws[2].wl_weights()
    assert int(h.sum()) == st.moves == 4 * 400 * c["n"]
    for s in ws:
        i = s.wl_info()
        parts = s.particles()
        box = s.box
        dx, dy = parts[0].pos[0] - parts[1].pos[0], parts[0].pos[1] - parts[1].pos[1]
        rx, ry = box[0] * (dx - np.rint(dx)), box[1] * (dy - np.rint(dy))
        assert i.currorder[0] == math.ceil((math.sqrt(rx * rx + ry * ry) - i.minorder[0]) / i.dorder[0])
    st, _, _, _, _ = R.run(20000, exchange_every=0, seed=5, variant=4)
    infos = [s.wl_info() for s in ws]
    assert len({(i.alpha, i.updates) for i in infos}) == 1          # one alpha for all walkers
    assert infos[0].updates >= 6, infos[0].updates
    w, _ = ws[0].wl_weights()
    assert np.array_equal(w, ws[3].wl_weights()[0])
    lo, hi = 2, 29
    ref = np.array([r["weights"] for r in c["ref_runs"]])[:, lo:hi]
    ref = (ref - ref.mean(1, keepdims=True)).mean(0)
    got = w[lo:hi] - w[lo:hi].mean()
    rms = float(np.sqrt(((got - ref) ** 2).mean()))
    assert rms < 0.45, (rms, np.round(got, 2), np.round(ref, 2))
    with pytest.raises(Exception):
        R.run(10, exchange_every=5, seed=6)                         # no exchange with weights
    R.close()
    for s in ws:
        s.close()


def test_run_stops_where_the_reference_stops(tmp_path):
    # alpha below WL_ALPHATOL and a histogram that is flat at the first check (10^9 visits
    # per bin): WangLandau::update reports convergence and the loop ends at that sweep
    s, c = open_case("o4_pair")
    lines = c["inputs"]["wl.dat"].splitlines()
    text = "5e-9\n" + "".join(f"{l.split()[0]} 0.0 1000000000\n" for l in lines[1:])
    s.wl_load(text=text)
    p = s.default_run()
    p.variant = 4
    st = s.simulate(p, nsweeps=5000, seed=33)
    i = s.wl_info()
    assert st.sweeps == 1000 and st.moves == 1000 * c["n"]
    assert i.converged == 1 and i.updates == 0 and i.alpha == 5e-9
    s.wl_end(tmp_path / "wl-new.dat")
    assert (tmp_path / "wl-new.dat").read_text().startswith(" 5.00000000e-09")
    s.close()
