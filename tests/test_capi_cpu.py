"""Host-side checks of the C ABI that need no GPU: the library loads, exports every
entry point of include/sc_gb300.h, and its readers of options / top.init /
config.init derive the reference's interaction table and particle vectors
bit-exactly (compared with goldens produced by the reference itself)."""
import ctypes as C
import os
import re

import pytest

import goldens

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from sc_gb300 import _lib
    from sc_gb300 import build as B

    B.build()
    return _lib.load()


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "sc_gb300.h")).read()
    return sorted(set(re.findall(r"\b(sc_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    from sc_gb300 import _lib

    assert sorted(n for n, _, _ in _lib.SIGNATURES) == syms


def test_every_entry_point_refuses_null_arguments(lib):
    """Every call given a NULL handle and NULL buffers (zero counts, zero sizes) returns an
    error code and leaves a message, instead of dereferencing them (the reference's calls
    exit the process on bad input; the C ABI never does).  sc_fp64_rates takes no handle and
    needs a GPU; destroying a NULL surrogate is a no-op, as free(NULL) is."""
    from sc_gb300 import _lib

    skip = {"sc_last_error", "sc_version", "sc_fp64_rates", "sc_surrogate_destroy"}
    checked = 0
    for name, _, argtypes in _lib.SIGNATURES:
        if name in skip:
            continue
        args = []
        for a in argtypes:
            if a in (C.c_int, C.c_long, C.c_ulonglong):
                args.append(0)
            elif a is C.c_double:
                args.append(0.0)
            else:
                args.append(None)
        rc = getattr(lib, name)(*args)
        assert rc < 0, (name, rc)
        assert lib.sc_last_error().decode(), name
        checked += 1
    assert checked >= 50
    assert lib.sc_surrogate_destroy(None) == 0


NAMES = goldens.names()


@pytest.mark.parametrize("name", NAMES)
def test_parsers_match_reference(lib, name):
    from sc_gb300 import System

    g = goldens.load(name)
    ref = g["ref"]
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    assert s.n == ref["n"]
    assert list(s.box) == ref["box"]
    sq, mc = s.cutoff()
    assert sq == ref["sqmaxcut"] and mc == ref["maxcut"]
    for e in ref["ia_params"]:
        p = s.pair_param(e["t1"], e["t2"])
        assert list(p.geotype) == e["geotype"]
        assert p.exclude == e["exclude"]
        for k in ("sigma", "epsilon", "A", "B", "pdis", "pswitch", "pswitchINV", "rcut", "rcutSq", "rcutwca",
                  "rcutwcaSq", "parallel"):
            assert getattr(p, k) == e[k], (k, e["t1"], e["t2"])
        if e["t1"] == e["t2"]:
            assert p.volume == e["volume"]
        for k in ("pcangl", "pcanglsw", "pcoshalfi", "psinhalfi", "csecpatchrot", "ssecpatchrot", "len", "half_len",
                  "chiral_cos", "chiral_sin"):
            assert list(getattr(p, k)) == e[k], (k, e["t1"], e["t2"])
    parts = s.particles()
    for q, d in zip(parts, ref["particles"]):
        assert list(q.pos) == d["pos"]
        assert list(q.dir) == d["dir"]
        for k in range(2):
            assert list(q.patchdir[k]) == d[f"pd{k}"]
            assert list(q.chdir[k]) == d[f"ch{k}"]
        # patchsides are set only for patchy spherocylinders (Particle::init); the
        # reference leaves the others uninitialised
        g0 = s.pair_param(d["type"], d["type"]).geotype[0]
        nsides = 0 if (g0 >= 30 or g0 in (10, 11)) else (4 if g0 in (16, 17, 18, 19) else 2)
        for k in range(nsides):
            assert list(q.patchsides[k]) == d[f"ps{k}"]
        assert q.type == d["type"] and q.molType == d["molType"]
    s.close()


def test_options_errors_are_reported_not_fatal(lib):
    from sc_gb300 import ScError, System

    g = goldens.load(NAMES[0])["inputs"]
    bad_opts = "\n".join(l for l in g["options"].splitlines() if not l.strip().startswith("temper"))
    with pytest.raises(ScError) as ei:
        System.from_text(bad_opts, g["top.init"], g["config.init"])
    assert "temper" in str(ei.value) and "PARSE" in str(ei.value)
    bad_top = g["top.init"].replace("PSC", "XPSC", 1)
    with pytest.raises(ScError):
        System.from_text(g["options"], bad_top, g["config.init"])
    short_cfg = "\n".join(g["config.init"].splitlines()[:5])
    with pytest.raises(ScError) as ei:
        System.from_text(g["options"], g["top.init"], short_cfg)
    assert "fewer particle lines" in str(ei.value)
    with pytest.raises(ScError):
        System.open("/nonexistent/options", "/nonexistent/top", "/nonexistent/config")


def test_moves_outside_the_gpu_loop_are_refused(lib):
    # the warp-per-cell kernel (variant bit 3) runs plain moves only: delayed acceptance with it
    # is refused before the device is touched
    from sc_gb300 import ScError, System

    g = goldens.load(NAMES[0])["inputs"]
    s = System.from_text(g["options"], g["top.init"], g["config.init"])
    with pytest.raises(ScError) as ei:
        s.simulate(nsweeps=1, variant=8, delayed=1)
    assert ei.value.code == -7 and "plain moves" in str(ei.value)
    s.close()


def test_write_config_format(lib, tmp_path):
    from sc_gb300 import System

    g = goldens.load("ref_test_01_normal_PSC")
    inp = g["inputs"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    path = str(tmp_path / "config.last")
    s.write_config(path)
    lines = open(path).read().splitlines()
    assert len(lines) == s.n + 1
    box = [float(x) for x in lines[0].split()]
    assert box == pytest.approx(list(s.box), rel=1e-8)
    fields = lines[1].split()
    assert len(fields) == 11
