"""Parity on the benchmark systems themselves, against the pinned oracle.

The goldens pin the GPU path on fixtures of at most a few hundred particles; these tests
take the seeded starts of the benchmark configurations -- 1000 PSC at packing fraction 0.1,
the 4000-particle CPSC + SPA mixture, 30,000 lipid beads with bonds, and 4096 targets of
65,536 PSC/CPSC at packing fraction 0.2 -- move them for a few GPU sweeps, hand the moved
state to the oracle, and compare:

  * every target's one-particle energy and (all targets) the total energy (|dE| <= 1e-12 of
    the sum of the absolute pair energies involved: the GPU sums in another order);
  * every pair PairE's prefilter admits (paire.h:1209-1215): verdict bits and closest
    segment distance^2 bit-exact, pair energy within 1e-12;
  * the move kernels' candidate screens (sc_screen_survivors): stage A keeps every non-bonded
    pair the prefilter admits, and every pair stage B drops has an exact energy of 0.
"""
import numpy as np
import pytest

import oracle_ffi as O

pytestmark = pytest.mark.gpu

CASES = {
    "nvt_psc_1000": (None, 10),
    "npt_cpsc_spa_4000": (None, 10),
    "bilayer_30000": (None, 4),
    "psc_cpsc_65536": (4096, 4),
}


def _bonded(ts, I, J):
    """Pairs bonded through the conlist (i +- 1 for bond1/bondd/bondh, i +- 2 for bond2 within
    one molecule), which the kernels evaluate whatever the screens say."""
    out = np.zeros(len(I), bool)
    for k in range(ts.sys.nmol):
        m = ts.mols[k]
        if m.size <= 1:
            continue
        lo, hi = m.first, m.first + m.size * m.count
        inside = (I >= lo) & (I < hi) & (J >= lo) & (J < hi)
        same = inside & ((I - lo) // m.size == (J - lo) // m.size)
        d = np.abs(I - J)
        b1 = (m.bond1c >= 0 or m.bonddc >= 0 or m.bondhc >= 0) & (d == 1)
        b2 = (m.bond2c >= 0) & (d == 2)
        out |= same & (b1 | b2)
    return out


@pytest.fixture(scope="module", params=list(CASES))
def moved(request):
    from sc_gb300 import System, workloads

    name = request.param
    ntarg, sweeps = CASES[name]
    texts = workloads.WORKLOADS[name](1)
    s = System.from_text(*texts)
    ts = O.TextSystem(*texts)
    s.simulate(nsweeps=sweeps, seed=7, check_every=0)
    ts.set_state(s.particles(), s.box)
    rng = np.random.default_rng(5)
    targets = np.arange(s.n, dtype=np.int32) if ntarg is None else np.sort(
        rng.choice(s.n, ntarg, replace=False)).astype(np.int32)
    I, J = ts.prefilter_pairs(targets)
    E, B, D = ts.pair_energies(I, J)
    yield name, s, ts, targets, (I, J, E, B, D)
    s.close()


def test_total_and_one_particle_energies(moved):
    name, s, ts, targets, (I, J, E, B, D) = moved
    e_gpu = s.one_to_all(targets)
    absum = np.zeros(s.n)
    np.add.at(absum, I, np.abs(E))
    worst = 0.0
    for k, t in enumerate(targets):
        want = ts.one_to_all(int(t))
        worst = max(worst, abs(e_gpu[k] - want) / max(1.0, absum[t]))
    assert worst <= 1e-12, (name, worst)
    if len(targets) == s.n:
        want = ts.all_to_all()
        got = s.all_to_all()
        assert abs(got - want) <= 1e-12 * max(1.0, 0.5 * float(np.abs(E).sum())), (name, got, want)


def test_prefilter_pairs_bit_exact(moved):
    name, s, ts, targets, (I, J, E, B, D) = moved
    Eg, Bg, Dg = s.pair_energies(I, J)
    assert np.array_equal(Bg, B), (name, int(np.sum(Bg != B)))
    assert np.array_equal(Dg, D), (name, int(np.sum(Dg != D)))
    assert np.all(np.abs(Eg - E) <= 1e-12 * np.maximum(1.0, np.abs(E))), name


def test_candidate_screens_cover_the_prefilter(moved):
    name, s, ts, targets, (I, J, E, B, D) = moved
    full = len(targets) == s.n
    Ia, Ja, Bs = s.screen_survivors(None if full else targets)
    keyA = Ia.astype(np.int64) * s.n + Ja
    # stage A keeps every non-bonded pair the prefilter admits
    nb = ~_bonded(ts, I, J)
    keyP = I[nb].astype(np.int64) * s.n + J[nb]
    missing = np.setdiff1d(keyP, keyA)
    assert len(missing) == 0, (name, len(missing), missing[:5])
    # every pair stage B drops has an exact energy of 0 (the oracle's, not the screen's)
    drop = Bs == 0
    assert drop.sum() > 0
    Ed, _, _ = ts.pair_energies(Ia[drop], Ja[drop])
    bonded = _bonded(ts, Ia[drop], Ja[drop])
    assert np.all(Ed[~bonded] == 0.0), (name, int(np.sum(Ed[~bonded] != 0.0)))


def test_nematic_order_matches_oracle(moved):
    """S2 and the director of the moved benchmark state: the GPU's fixed-order reduction and
    the oracle's sums agree to rounding."""
    name, s, ts, targets, _ = moved
    s2, d = s.nematic_order()
    s2o, do = ts.nematic()
    assert abs(s2 - s2o) <= 1e-12, (name, s2, s2o)
    assert abs(abs(float(np.dot(d, do))) - 1.0) <= 1e-9 or s2 < 1e-3, (name, d, do)
