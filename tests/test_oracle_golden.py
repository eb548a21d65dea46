"""Pins the CPU oracle to golden vectors produced by the reference itself.

Energies within 1e-12 relative (of max(|E|, sum|e_ij|)), verdict bits bit-exact,
derived parameters and derived particle vectors bit-exact.
"""
import ctypes as C
import math

import pytest

import goldens
import oracle_ffi as O

NAMES = goldens.names()
REL = 1e-12


def close(a, b, scale):
    if math.isinf(a) or math.isinf(b) or math.isnan(a) or math.isnan(b):
        return (a == b) or (math.isnan(a) and math.isnan(b))
    return abs(a - b) <= REL * max(abs(scale), abs(a), abs(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_pair_energies_and_verdicts(name):
    g = goldens.load(name)
    ref = g["ref"]
    s = O.OracleSystem(ref)
    listed = set()
    bad = []
    for i, j, e, bits, dsq in ref["pairs"]:
        listed.add((i, j))
        eo, bo, do = s.pair(i, j)
        if bo != bits:
            bad.append(("bits", i, j, bits, bo))
        if not close(eo, e, e):
            bad.append(("energy", i, j, e, eo))
        if dsq >= 0 and do != dsq:
            bad.append(("distSq", i, j, dsq, do))
    assert not bad, bad[:10]
    # every pair not listed was prefiltered by the reference: energy exactly 0, no EVAL bit
    n = ref["n"]
    step = max(1, (n * n) // 20000)
    for k in range(0, n * n, step):
        i, j = divmod(k, n)
        if i == j or (i, j) in listed:
            continue
        eo, bo, _ = s.pair(i, j)
        assert eo == 0.0 and bo == 0, (i, j, eo, bo)


@pytest.mark.parametrize("name", NAMES)
def test_one_to_all_all_to_all(name):
    ref = goldens.load(name)["ref"]
    s = O.OracleSystem(ref)
    sabs = sum(abs(p[2]) for p in ref["pairs"])
    for i, e in enumerate(ref["one_to_all"]):
        assert close(s.one_to_all(i), e, sabs), (i, e)
    assert close(s.all_to_all(), ref["all_to_all"], sabs)
    for first, size, e in ref["mol2others"]:
        assert close(s.mol2others(first, size), e, sabs)


@pytest.mark.parametrize("name", NAMES)
def test_trial_moves(name):
    ref = goldens.load(name)["ref"]
    s = O.OracleSystem(ref)
    sabs = sum(abs(p[2]) for p in ref["pairs"])
    for tr in ref["trials"]:
        t = tr["target"]
        orig = O.particle_from_ref(ref["particles"][t])
        p = O.particle_from_ref(ref["particles"][t])
        if tr["displace"]:
            p.pos.x += tr["dr"][0]
            p.pos.y += tr["dr"][1]
            p.pos.z += tr["dr"][2]
        else:
            g0 = s.params[p.type * O.MAXT + p.type].geotype[0]
            O.lib().or_psc_rotate(C.byref(p), g0, tr["angle"], O.vec(tr["axis"]), tr["cw"])
            # partRotate re-orthogonalises patchdir[0] (movecreator.cpp:1007)
            d = p.dir
            dp = p.pd[0].x * d.x + p.pd[0].y * d.y + p.pd[0].z * d.z
            p.pd[0].x -= dp * d.x
            p.pd[0].y -= dp * d.y
            p.pd[0].z -= dp * d.z
        st = tr["state"]
        for key, v in (("pos", p.pos), ("dir", p.dir), ("pd0", p.pd[0]), ("pd1", p.pd[1]), ("ps0", p.ps[0]),
                       ("ps1", p.ps[1]), ("ps2", p.ps[2]), ("ps3", p.ps[3]), ("ch0", p.ch[0]), ("ch1", p.ch[1])):
            assert [v.x, v.y, v.z] == st[key], (key, t)
        assert close(s.one_to_all(t), tr["e_old"], sabs)
        s.parts[t] = p
        assert close(s.one_to_all(t), tr["e_new"], sabs)
        s.parts[t] = orig


@pytest.mark.parametrize("name", NAMES)
def test_volume_trials(name):
    ref = goldens.load(name)["ref"]
    s = O.OracleSystem(ref)
    sabs = sum(abs(p[2]) for p in ref["pairs"])
    box = list(ref["box"])
    for vt in ref["volume_trials"]:
        for k in range(3):
            s.sys.box[k] = box[k] + vt["psch"]
        assert close(s.all_to_all(), vt["e_new"], sabs)
        for k in range(3):
            s.sys.box[k] = box[k]


@pytest.mark.parametrize("name", NAMES)
def test_derived_parameters_and_particles(name):
    g = goldens.load(name)
    ref = g["ref"]
    types, excl = O.parse_types(g["inputs"]["top.init"])
    arr = (O.TypeIn * len(types))(*types)
    table = (O.Param * (O.MAXT * O.MAXT))()
    sq, mc = C.c_double(), C.c_double()
    rc = O.lib().or_derive_params(arr, len(types), excl.ctypes.data, table, C.byref(sq), C.byref(mc))
    assert rc == 0
    assert sq.value == ref["sqmaxcut"] and mc.value == ref["maxcut"]
    want = O.params_from_ref(ref)
    for e in ref["ia_params"]:
        a, b = table[e["t1"] * O.MAXT + e["t2"]], want[e["t1"] * O.MAXT + e["t2"]]
        for fld, _ in O.Param._fields_:
            if fld in ("pad_", "volume") and (fld == "pad_" or e["t1"] != e["t2"]):
                continue
            va, vb = getattr(a, fld), getattr(b, fld)
            if hasattr(va, "__len__"):
                va, vb = list(va), list(vb)
            assert va == vb, (e["t1"], e["t2"], fld, va, vb)
    # Particle::init (via Conf::partVecInit) on the particles as initConfig left them
    for d_in, d in zip(ref["particles_in"], ref["particles"]):
        p = O.particle_from_ref(d_in)
        diag = want[p.type * O.MAXT + p.type]
        if diag.geotype[0] < 30:     # partVecInit skips spheres (Conf.cpp:97-102)
            O.lib().or_particle_init(C.byref(p), C.byref(diag))
        q = O.particle_from_ref(d)
        for name, u, v in [("dir", p.dir, q.dir)] + [(f"pd{k}", p.pd[k], q.pd[k]) for k in range(2)] + \
                [(f"ps{k}", p.ps[k], q.ps[k]) for k in range(4)] + [(f"ch{k}", p.ch[k], q.ch[k]) for k in range(2)]:
            assert [u.x, u.y, u.z] == [v.x, v.y, v.z], name
