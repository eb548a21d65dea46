"""The CPU baseline: the oracle's own set-up of a system from the reference's inputs, its
resumable sequential loop, and its timing against the reference's own -Ofast build.

The bench times the reference's algorithm on the GPU host's cores with the oracle's
restatement (oracle/sc_oracle.cpp, built at the reference's -Ofast by oracle/Makefile),
because the reference binary built here does not run there.  These tests pin that
stand-in: it reads the same texts as the GPU path (same particles), keeps its running
energy exact in both energy-calculator modes (TotalEMatrix and TotalEFull), and runs within
15 % of the reference's own -Ofast binary on 10 sweeps of the 4000-particle NPT mixture.
"""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import oracle_ffi as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SC_REF_FAST = os.path.join(ROOT, "oracle", "_ref", "sc_ref_fast")


def _texts(name):
    from sc_gb300 import workloads

    if name == "mixture":
        return workloads.npt_cpsc_spa(400, seed=3)
    if name == "lipids":
        return workloads.lipids_dilute(24, seed=2)
    return workloads.psc_cpsc(2048, phi=0.2, seed=4)


@pytest.mark.parametrize("name", ["mixture", "lipids", "psc_cpsc"])
def test_oracle_setup_matches_library_parse(name):
    """The oracle's set-up of options / top.init / config.init gives the particles the GPU
    library's parser gives (positions, axes, patch vectors), without the GPU library."""
    from sc_gb300 import System

    texts = _texts(name)
    ts = O.TextSystem(*texts)
    s = System.from_text(*texts)
    parts = s.particles()
    assert ts.sys.n == s.n
    assert np.array_equal(list(ts.sys.box), s.box)
    worst = 0.0
    for k in range(s.n):
        a, b = parts[k], ts.parts[k]
        assert a.type == b.type and a.molType == b.molType
        pairs = [(a.pos, b.pos), (a.dir, b.dir), (a.patchdir[0], b.pd[0]), (a.patchdir[1], b.pd[1])]
        pairs += [(a.patchsides[m], b.ps[m]) for m in range(4)] + [(a.chdir[m], b.ch[m]) for m in range(2)]
        for u, v in pairs:
            worst = max(worst, max(abs(u[0] - v.x), abs(u[1] - v.y), abs(u[2] - v.z)))
    assert worst <= 4e-16, worst
    s.close()


@pytest.mark.parametrize("matrix", [True, False])
def test_resumable_loop_keeps_energy_exact(matrix):
    """or_mc_open / or_mc_advance in pieces: the running energy equals the exact total after
    moves, pair-list rebuilds and volume moves, in both energy-calculator modes."""
    texts = _texts("mixture")
    ts = O.TextSystem(*texts)
    run = O.McRun(ts, seed=9, energy_matrix=matrix)
    n = ts.sys.n
    for chunk in (1, 7, n, 3 * n + 5, 12 * n):
        st = run.advance(chunk)
    assert st.moves == 1 + 7 + n + 3 * n + 5 + 12 * n
    assert st.acc_trans + st.acc_rot > 0 and st.acc_vol + st.rej_vol > 0
    exact = ts.all_to_all()
    assert abs(run.energy - exact) <= 1e-9 * max(1.0, abs(exact)), (run.energy, exact)
    run.close()


def _ref_seconds(texts, tmp):
    opts, top, cfg = texts
    for name, t in (("options", opts), ("top.init", top), ("config.init", cfg)):
        with open(os.path.join(tmp, name), "w") as f:
            f.write(t)
    r = subprocess.run([SC_REF_FAST], cwd=tmp, capture_output=True, text=True, check=True)
    m = re.findall(r"Simulation time:\s*([0-9.eE+-]+)\s*s", r.stdout)
    assert m, r.stdout[-400:]
    return float(m[-1])


@pytest.mark.skipif(not os.path.exists(SC_REF_FAST), reason="the reference's -Ofast build (oracle/_ref) is absent")
def test_fast_port_runs_at_the_reference_speed():
    """10 sweeps of the 4000-particle NPT mixture (pair list every 10 sweeps, one volume move
    per sweep on average, the reference's energy matrix): the -Ofast port within 15 % of the
    reference's own -Ofast binary (best of two runs each, the reference's own timer)."""
    from sc_gb300 import workloads

    opts, top, cfg = workloads.npt_cpsc_spa(4000, seed=1)
    d = O.parse_options(opts)
    d.update(nsweeps="10", report="1000", movie="0", nequil="0", pairlist_update="10")
    opts = "".join(f"{k} = {v}\n" for k, v in d.items())
    ref, port = [], []
    for _ in range(2):
        with tempfile.TemporaryDirectory() as tmp:
            ref.append(_ref_seconds((opts, top, cfg), tmp))
        ts = O.TextSystem(opts, top, cfg)
        run = O.McRun(ts, energy_matrix=True, fast=True)
        port.append(run.advance(10 * ts.sys.n).seconds)
        run.close()
    ratio = min(port) / min(ref)
    assert 0.85 <= ratio <= 1.15, (port, ref)
