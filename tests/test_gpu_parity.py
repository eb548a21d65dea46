"""GPU parity: the CUDA energy path against the reference's own numbers.

Every call goes through the C ABI (libscgpu.so).  Verdict bits and closest segment
distances must be bit-identical, energies within 1e-12 relative of
max(|E|, sum |e_ij|), trial states bit-identical.
"""
import math

import numpy as np
import pytest

import goldens

pytestmark = pytest.mark.gpu
NAMES = goldens.names()
REL = 1e-12


def close(a, b, scale):
    if not (math.isfinite(a) and math.isfinite(b)):
        return a == b or (math.isnan(a) and math.isnan(b))
    return abs(a - b) <= REL * max(abs(scale), abs(a), abs(b), 1e-300)


def open_golden(name):
    from sc_gb300 import System

    g = goldens.load(name)
    inp = g["inputs"]
    return g["ref"], System.from_text(inp["options"], inp["top.init"], inp["config.init"])


@pytest.mark.parametrize("name", NAMES)
def test_pair_energies_verdicts(name):
    ref, s = open_golden(name)
    P = np.array([p[:2] for p in ref["pairs"]], dtype=np.int32).reshape(-1, 2)
    E, V, D = s.pair_energies(P[:, 0], P[:, 1])
    bad = []
    for k, (i, j, e, bits, dsq) in enumerate(ref["pairs"]):
        if V[k] != bits:
            bad.append(("bits", i, j, bits, int(V[k])))
        if dsq >= 0 and D[k] != dsq:
            bad.append(("distSq", i, j, dsq, D[k]))
        # a pair energy is a sum of O(epsilon) terms (WCA, attraction, bonds): the
        # tolerance is 1e-12 of max(|E|, 1 kT)
        if not close(E[k], e, max(abs(e), 1.0)):
            bad.append(("energy", i, j, e, E[k]))
    assert not bad, bad[:10]
    # pairs the reference prefiltered: exactly zero, no verdict
    n = ref["n"]
    listed = set(map(tuple, P.tolist()))
    rest = [(i, j) for i in range(n) for j in range(n) if i != j and (i, j) not in listed]
    if rest:
        R = np.array(rest, dtype=np.int32)
        E2, V2, _ = s.pair_energies(R[:, 0], R[:, 1])
        assert np.all(E2 == 0.0) and np.all(V2 == 0)
    s.close()


@pytest.mark.parametrize("name", NAMES)
def test_one_to_all_all_to_all(name):
    ref, s = open_golden(name)
    sabs = sum(abs(p[2]) for p in ref["pairs"])
    got = s.one_to_all(np.arange(ref["n"]))
    for i, e in enumerate(ref["one_to_all"]):
        assert close(got[i], e, sabs), (i, got[i], e)
    assert close(s.all_to_all(), ref["all_to_all"], sabs)
    for first, size, e in ref["mol2others"]:
        assert close(s.mol2others(first, size), e, sabs)
    s.close()


@pytest.mark.parametrize("name", NAMES)
def test_trial_moves(name):
    ref, s = open_golden(name)
    sabs = sum(abs(p[2]) for p in ref["pairs"])
    for tr in ref["trials"]:
        t = tr["target"]
        st = tr["state"]
        if tr["displace"]:
            eo, en = s.trial_displace(t, tr["dr"])
            pos = [ref["particles"][t]["pos"][k] + tr["dr"][k] for k in range(3)]
            assert pos == st["pos"]
        else:
            eo, en, q = s.trial_rotate(t, tr["angle"], tr["axis"], tr["cw"])
            assert list(q.dir) == st["dir"]
            assert list(q.patchdir[0]) == st["pd0"] and list(q.patchdir[1]) == st["pd1"]
            g0 = s.pair_param(q.type, q.type).geotype[0]
            nsides = 0 if (g0 >= 30 or g0 in (10, 11)) else (4 if g0 in (16, 17, 18, 19) else 2)
            for k in range(nsides):
                assert list(q.patchsides[k]) == st[f"ps{k}"]
            assert list(q.chdir[0]) == st["ch0"] and list(q.chdir[1]) == st["ch1"]
        assert close(eo, tr["e_old"], sabs)
        assert close(en, tr["e_new"], sabs)
    s.close()


@pytest.mark.parametrize("name", NAMES)
def test_volume_trials(name):
    ref, s = open_golden(name)
    sabs = sum(abs(p[2]) for p in ref["pairs"])
    for vt in ref["volume_trials"]:
        assert close(s.trial_volume(vt["psch"]), vt["e_new"], sabs)
    s.close()


def test_accept_trial_updates_state():
    ref, s = open_golden("syn_psc_nvt_small")
    t = ref["trials"][0]["target"]
    dr = [0.01, -0.02, 0.005]
    eo, en = s.trial_displace(t, dr)
    s.accept_trial()
    e2 = s.one_to_all([t])[0]
    assert e2 == pytest.approx(en, rel=1e-12, abs=1e-12)
    q = s.particles(t, 1)[0]
    assert list(q.pos) == [ref["particles"][t]["pos"][k] + dr[k] for k in range(3)]
    s.close()
