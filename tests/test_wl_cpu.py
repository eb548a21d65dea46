"""Wang-Landau without a GPU: the weights file, the starting bins and the system centre.

The goldens (tests/golden/wl/cases.json.gz, made by tests/golden/make_wl.py) hold what the
reference itself computes with its WangLandau::init and writes with WangLandau::write
(scOOP/mc/wanglandau.cpp:49-166) for seeded systems and weights files.  Both the oracle's
restatement (or_wl_orders) and the library's host code (sc_wl_load / sc_wl_get_info /
sc_wl_write, which run before any device work) must reproduce them exactly.  The oracle's
sequential Wang-Landau loop (or_wl_run) is checked against the reference's own adaptive runs.
The cases include the reference's own membrane test (a CPSC protein and 200 lipids, orders 1
and 3) with the converged weights of its legacy run as the weights file.
"""
import gzip
import json
import os

import pytest

import oracle_ffi as O

HERE = os.path.dirname(os.path.abspath(__file__))
WL_GOLDEN = os.path.join(HERE, "golden", "wl", "cases.json.gz")
ERR_STATE, ERR_UNSUPPORTED, ERR_RANGE, ERR_PARSE = -6, -7, -5, -3


def cases():
    with gzip.open(WL_GOLDEN, "rt") as f:
        return json.load(f)["cases"]


CASES = cases()


@pytest.fixture(scope="module")
def System():
    from sc_gb300 import System as S
    from sc_gb300 import build as B

    B.build()
    return S


def wlm_of(c):
    for line in c["inputs"]["options"].splitlines():
        k, _, v = line.partition("=")
        if k.strip() == "wlm":
            w = [int(x) for x in v.split("#")[0].split()]
            return (w + [0])[:2]
    raise KeyError("wlm")


def wlmtype_of(c):
    for line in c["inputs"]["options"].splitlines():
        k, _, v = line.partition("=")
        if k.strip() == "wlmtype":
            return int(v.split("#")[0].split()[0])
    return -1


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_oracle_starting_bins_match_reference(c):
    ref = c["ref"]
    o = O.OracleSystem(c["system"])
    rc, bins, cm, sv = o.wl_orders(wlm_of(c), ref["minorder"], ref["dorder"], wlmtype_of(c))
    assert rc == 0
    dim = 2 if wlm_of(c)[1] else 1
    assert bins[:dim] == ref["currorder"][:dim]
    assert sv == ref["sysvolume"]
    if 1 in wlm_of(c):                      # the reference computes the centre for order 1 only
        assert cm == ref["syscm"]


@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_library_loads_weights_like_the_reference(System, c, tmp_path):
    inp = c["inputs"]
    ref = c["ref"]
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    if 2 in wlm_of(c):                      # the mesh hole: the oracle's only
        from sc_gb300._lib import ScError

        with pytest.raises(ScError) as e:
            s.wl_load(text=inp["wl.dat"])
        assert e.value.code == ERR_UNSUPPORTED
        s.close()
        return
    s.wl_load(text=inp["wl.dat"])
    i = s.wl_info()
    dim = 2 if wlm_of(c)[1] else 1
    assert i.dim == dim
    assert [i.length[0], i.length[1]] == ref["length"]
    assert [i.currorder[0], i.currorder[1]][:dim] == ref["currorder"][:dim]
    assert i.alpha == ref["alpha"]
    assert [i.minorder[0], i.minorder[1]][:dim] == ref["minorder"][:dim]
    assert [i.dorder[0], i.dorder[1]][:dim] == ref["dorder"][:dim]
    if 1 in wlm_of(c):
        assert [i.syscm[0], i.syscm[1], i.syscm[2]] == ref["syscm"]
    # WangLandau::write of the weights just read: the same text
    out = tmp_path / "wl-out.dat"
    s.wl_write(out)
    assert out.read_text() == ref["written"]
    s.close()


def test_open_reads_wl_dat_beside_the_options(System, tmp_path):
    c = CASES[0]
    for fn in ("options", "top.init", "config.init", "wl.dat"):
        (tmp_path / fn).write_text(c["inputs"][fn])
    s = System.open(tmp_path / "options", tmp_path / "top.init", tmp_path / "config.init")
    assert s.wl_info().currorder[0] == c["ref"]["currorder"][0]
    s.close()


def test_end_shifts_two_dimensional_weights_only(System, tmp_path):
    for c in CASES:
        if 2 in wlm_of(c):
            continue
        inp = c["inputs"]
        s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
        s.wl_load(text=inp["wl.dat"])
        w, _ = s.wl_weights()
        s.wl_end(tmp_path / "end.dat")
        rows = [l.split() for l in (tmp_path / "end.dat").read_text().splitlines()[1:] if l.strip()]
        got = [float(r[-2]) for r in rows]
        want = (w - w[0]) if s.wl_info().dim == 2 else w
        assert got == pytest.approx(list(want), abs=1e-7, rel=1e-7)
        s.close()


def _sub(text, key, value):
    out = []
    for line in text.splitlines():
        if line.split("=")[0].strip() == key:
            line = f"{key} = {value}"
        out.append(line)
    return "\n".join(out) + "\n"


def test_rejections(System):
    from sc_gb300._lib import ScError

    c = next(c for c in CASES if c["name"] == "o4_pair")
    inp = c["inputs"]
    # the mesh-hole and pore order parameters are not on the GPU path
    for m in (2, 5, 6):
        s = System.from_text(_sub(inp["options"], "wlm", f"{m} 0"), inp["top.init"], inp["config.init"])
        with pytest.raises(ScError) as e:
            s.wl_load(text=inp["wl.dat"])
        assert e.value.code == ERR_UNSUPPORTED
        s.close()
    # a starting bin outside the file's range
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    lines = inp["wl.dat"].splitlines()
    short = "\n".join(lines[:4]) + "\n"           # alpha + three bins below the start
    with pytest.raises(ScError) as e:
        s.wl_load(text=short)
    assert e.value.code == ERR_RANGE
    # two order parameters in the options, one in the file
    s2 = System.from_text(_sub(inp["options"], "wlm", "4 8"), inp["top.init"], inp["config.init"])
    with pytest.raises(ScError) as e:
        s2.wl_load(text=inp["wl.dat"])
    assert e.value.code == ERR_PARSE
    # wlm > 0 and no weights: the move loop refuses before touching the device
    with pytest.raises(ScError) as e:
        s.simulate(nsweeps=1)
    assert e.value.code == ERR_STATE
    s.close()
    s2.close()


def test_oracle_wang_landau_run_matches_the_reference_runs():
    # or_wl_run (the oracle's sequential loop with the bias) on the two-particle distance
    # case: its adaptive weights match the reference's own runs of the same system
    import numpy as np

    c = next(c for c in CASES if c["name"] == "o4_pair")
    ref = c["ref"]
    o = O.OracleSystem(c["system"])
    opts = O.McOpts()
    opts.nsweeps, opts.seed, opts.temper = 60000, 7, 1.0
    opts.transmx = 0.6                    # options transmx 0.3, doubled as sim.h:365 does
    nb = ref["length"][0]
    w, h, st, ms = o.wl_run(opts, (4, 0), ref["minorder"], ref["dorder"], (nb, 1), ref["alpha"],
                            np.zeros(nb), np.zeros(nb, dtype=np.int64))
    assert ms.moves == 60000 * c["n"]
    assert st.updates >= 8, st.updates
    lo, hi = 2, 29
    R = np.array([r["weights"] for r in c["ref_runs"]])[:, lo:hi]
    R = (R - R.mean(1, keepdims=True)).mean(0)
    got = w[lo:hi] - w[lo:hi].mean()
    rms = float(np.sqrt(((got - R) ** 2).mean()))
    assert rms < 0.25, (rms, np.round(got, 2), np.round(R, 2))


def test_share_checks_its_walkers(System):
    from sc_gb300._lib import ScError

    a = next(c for c in CASES if c["name"] == "o4_pair")
    b = next(c for c in CASES if c["name"] == "o1_bath")
    sa = System.from_text(a["inputs"]["options"], a["inputs"]["top.init"], a["inputs"]["config.init"])
    sb = System.from_text(b["inputs"]["options"], b["inputs"]["top.init"], b["inputs"]["config.init"])
    with pytest.raises(ScError) as e:
        System.wl_share([sa, sb])                  # no weights loaded yet
    assert e.value.code == ERR_STATE
    sa.wl_load(text=a["inputs"]["wl.dat"])
    sb.wl_load(text=b["inputs"]["wl.dat"])
    with pytest.raises(ScError) as e:
        System.wl_share([sa, sb])                  # other order parameters and bins
    assert e.value.code == -1
    s2 = System.from_text(a["inputs"]["options"], a["inputs"]["top.init"], a["inputs"]["config.init"])
    s2.wl_load(text=a["inputs"]["wl.dat"])
    System.wl_share([sa, s2])                      # same bins: one table
    assert s2.wl_info().currorder[0] == sa.wl_info().currorder[0]
    for s in (sa, sb, s2):
        s.close()


def test_oracle_fixed_weights_bias_like_the_reference():
    # fixed weights w = 1.5 o of particle 0's axis z component: the oracle's loop and the
    # reference's own runs both give a histogram ln H = w / T + c (T = 1)
    import math

    import numpy as np

    c = next(c for c in CASES if c["name"] == "o3_orient")
    ref = c["ref"]
    o = O.OracleSystem(c["system"])
    opts = O.McOpts()
    opts.nsweeps, opts.seed, opts.temper = 50000, 11, 1.0
    opts.transmx = 0.4                          # options transmx 0.2, doubled (sim.h:365)
    opts.rot_angle = 120.0 / 180.0 * math.pi / 2 * 0.5     # rotmx 120 (sim.h:359)
    nb = ref["length"][0]
    orders = -1.0 + 0.05 * np.arange(nb)
    w, h, st, ms = o.wl_run(opts, (3, 0), ref["minorder"], ref["dorder"], (nb, 1), 0.0, 1.5 * orders,
                            np.zeros(nb, dtype=np.int64))
    assert st.updates == 0 and np.array_equal(w, 1.5 * orders)

    def slope(hist):
        hist = np.asarray(hist, float)[:40]
        sel = hist > 0
        return np.polyfit(orders[:40][sel], np.log(hist[sel]), 1, w=np.sqrt(hist[sel]))[0]

    mine = slope(h)
    theirs = [slope(r["hist"]) for r in c["ref_runs"]]
    assert abs(mine - 1.5) < 0.2, mine
    assert abs(mine - float(np.mean(theirs))) < 0.35, (mine, theirs)


def test_weights_file_reader_follows_init_calc(System):
    # WangLandau::initCalc: '#' comments and blank lines are skipped, alpha comes first, a
    # grid of two order parameters needs whole rows; a negligible alpha means fixed weights
    from sc_gb300._lib import ScError

    c = next(c for c in CASES if c["name"] == "o4_pair")
    inp = c["inputs"]
    lines = inp["wl.dat"].splitlines()
    noisy = "# weights\n\n" + lines[0] + "   # alpha\n" + "\n".join(l + "  # bin" for l in lines[1:]) + "\n\n"
    s = System.from_text(inp["options"], inp["top.init"], inp["config.init"])
    s.wl_load(text=noisy)
    i = s.wl_info()
    assert i.length[0] == len(lines) - 1 and i.currorder[0] == c["ref"]["currorder"][0]
    s.wl_load(text="1e-11\n" + "\n".join(lines[1:]) + "\n")
    assert s.wl_info().alpha == 0.0                     # below WL_ALPHATOL / 100
    for bad in ("", "x\n0 0 0\n", lines[0] + "\n0.1 0 0\n", lines[0] + "\n0.1 0\n0.2 0\n"):
        with pytest.raises(ScError) as e:
            s.wl_load(text=bad)
        assert e.value.code == ERR_PARSE
    s.close()
    d = next(c for c in CASES if c["name"] == "o8_o9")
    rows = d["inputs"]["wl.dat"].splitlines()
    s = System.from_text(d["inputs"]["options"], d["inputs"]["top.init"], d["inputs"]["config.init"])
    with pytest.raises(ScError) as e:
        s.wl_load(text="\n".join(rows[:-1]) + "\n")     # the last row one bin short
    assert e.value.code == ERR_PARSE
    s.close()


def test_oracle_volume_moves_respect_a_weight_wall_like_the_reference():
    # fixed weights 0 inside bins 5..15 of the box length in y and -1e4 outside (ptype 5:
    # only y changes): neither the reference nor the oracle's loop ever enters the wall,
    # and both pile up against its upper side (no pressure: the box wants to grow)
    import numpy as np

    c = next(c for c in CASES if c["name"] == "o9_wall")
    ref = c["ref"]
    o = O.OracleSystem(c["system"])
    opts = O.McOpts()
    opts.nsweeps, opts.seed, opts.temper, opts.press = 3000, 5, 1.0, 0.0
    opts.transmx, opts.edge_mx, opts.shave, opts.ptype = 0.4, 0.2, 1.0, 5   # options values doubled (sim.h:363-365)
    nb = ref["length"][0]
    w0 = np.array([0.0 if 5 <= k <= 15 else -1e4 for k in range(nb)])
    w, h, st, ms = o.wl_run(opts, (9, 0), ref["minorder"], ref["dorder"], (nb, 1), 0.0, w0,
                            np.zeros(nb, dtype=np.int64))
    theirs = np.array(c["ref_runs"][0]["hist"])
    for hist in (h, theirs):
        assert hist[:5].sum() == 0 and hist[16:].sum() == 0
        assert hist[15] > hist[5]
    assert int(h.sum()) == ms.moves == 3000 * c["n"]
    assert ms.acc_vol > 0 and ms.rej_vol > 0


@pytest.mark.parametrize("ptype", [3, 4])
def test_oracle_wl_loop_with_couplings_3_and_4(ptype):
    # the same wall on the box length in y under the two couplings restated last: ptype 4
    # (the reference's x-or-y test always takes x) never changes y, so every visit stays in
    # the starting bin; ptype 3 changes x and y together at constant volume, so y moves
    # between bins but never into the wall, and the volume stays what it was
    import numpy as np

    c = next(c for c in CASES if c["name"] == "o9_wall")
    ref = c["ref"]
    o = O.OracleSystem(c["system"])
    v0 = o.sys.box[0] * o.sys.box[1] * o.sys.box[2]
    y0 = o.sys.box[1]
    opts = O.McOpts()
    opts.nsweeps, opts.seed, opts.temper, opts.press = 3000, 7, 1.0, 0.0
    opts.transmx, opts.edge_mx, opts.shave, opts.ptype = 0.4, 0.2, 1.0, ptype
    nb = ref["length"][0]
    w0 = np.array([0.0 if 5 <= k <= 15 else -1e4 for k in range(nb)])
    w, h, st, ms = o.wl_run(opts, (9, 0), ref["minorder"], ref["dorder"], (nb, 1), 0.0, w0,
                            np.zeros(nb, dtype=np.int64))
    assert int(h.sum()) == ms.moves == 3000 * c["n"]
    assert ms.acc_vol > 0 and ms.rej_vol > 0
    assert h[:5].sum() == 0 and h[16:].sum() == 0
    if ptype == 4:
        assert np.count_nonzero(h) == 1 and o.sys.box[1] == y0
    else:
        assert np.count_nonzero(h) > 3
        assert abs(o.sys.box[0] * o.sys.box[1] * o.sys.box[2] - v0) <= 1e-12 * v0


def _options(c):
    d = {}
    for line in c["inputs"]["options"].splitlines():
        k, _, v = line.partition("=")
        if k.strip():
            d[k.strip()] = v.split("#")[0].strip()
    return d


@pytest.mark.parametrize("name", ["o7_contact", "o7_npt", "o2_mesh"])
def test_oracle_contact_and_mesh_orders_match_the_reference_runs(name):
    # the contact count (order 7; with volume moves that recount it in the trial box) and the
    # largest mesh hole (order 2) under fixed weights linear in the bin: twelve runs of the
    # oracle's loop and six of the reference's own give the same mean bin (3 combined standard
    # errors) and the same spread
    import math

    import numpy as np

    c = next(c for c in CASES if c["name"] == name)
    ref = c["ref"]
    d = _options(c)
    nb = ref["length"][0]
    w0 = np.array([float(l.split()[1]) for l in c["inputs"]["wl.dat"].splitlines()[1:] if l.strip()])
    means, sds = [], []
    for seed in range(1, 13):
        o = O.OracleSystem(c["system"])
        opts = O.McOpts()
        opts.nsweeps, opts.seed, opts.temper = int(d["nsweeps"]), seed, float(d["temper"])
        opts.transmx = 2.0 * float(d["transmx"])              # doubled as sim.h:363-365 does
        opts.shave, opts.ptype, opts.press = float(d["shave"]), int(d["ptype"]), float(d["press"])
        opts.edge_mx = 2.0 * float(d["edge_mx"])
        w, h, st, ms = o.wl_run(opts, (wlm_of(c)[0], 0), ref["minorder"], ref["dorder"], (nb, 1), 0.0, w0,
                                np.zeros(nb, dtype=np.int64), wlmtype=wlmtype_of(c))
        assert np.array_equal(w, w0) and int(h.sum()) == ms.moves == int(d["nsweeps"]) * c["n"]
        if opts.shave > 0:
            assert ms.acc_vol > 0 and ms.rej_vol > 0
        k = np.arange(nb)
        m = float((k * h).sum() / h.sum())
        means.append(m)
        sds.append(math.sqrt(float((h * (k - m) ** 2).sum() / h.sum())))
    theirs = []
    their_sd = []
    for r in c["ref_runs"]:
        h = np.array(r["hist"], float)
        k = np.arange(nb)
        m = float((k * h).sum() / h.sum())
        theirs.append(m)
        their_sd.append(math.sqrt(float((h * (k - m) ** 2).sum() / h.sum())))
    a, b = np.array(means), np.array(theirs)
    se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    print(name, "mean bin: oracle", a.mean(), "reference", b.mean(), "se", se, "sd", np.mean(sds), np.mean(their_sd))
    assert abs(a.mean() - b.mean()) <= 3.0 * se, (means, theirs)
    assert abs(np.mean(sds) - np.mean(their_sd)) <= 0.25 * np.mean(their_sd), (sds, their_sd)


def test_reference_pore_orders_end_at_init():
    # the pore orders 5 and 6: the reference's WangLandau::radiusholeAll
    # (scOOP/mc/wanglandau.cpp:306-318) declares a local radiusholemax that hides the member,
    # never allocates the histogram and writes through the null pointer init left, so the
    # reference's own main ends with SIGSEGV at WangLandau::init; there is no run to match
    import shutil
    import subprocess
    import tempfile

    exe = os.path.join(HERE, "..", "oracle", "_ref", "sc_ref")
    if not os.path.exists(exe):
        pytest.skip("the reference's build (oracle/_ref) is absent")
    c = next(c for c in CASES if c["name"] == "o1_bath")
    rows = "".join("%g 0 0\n" % (0.1 * k) for k in range(100))
    for m in (5, 6):
        d = tempfile.mkdtemp()
        try:
            opts = _sub(_sub(_sub(c["inputs"]["options"], "wlm", f"{m} 0"), "wlmtype", "2"), "nsweeps", "10")
            for fn, text in (("options", opts), ("top.init", c["inputs"]["top.init"]),
                             ("config.init", c["inputs"]["config.init"]), ("wl.dat", "0.1\n" + rows)):
                with open(os.path.join(d, fn), "w") as f:
                    f.write(text)
            r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=120)
            assert r.returncode == -11, (m, r.returncode, r.stdout[-300:])
            assert "Wang-Landau method init" in r.stdout
        finally:
            shutil.rmtree(d)


def test_contact_order_refuses_chain_moves_of_counted_chains(System):
    # order 7 with chain moves: chains that hold particles of type wlmtype would change the
    # count outside the cells moved in sequence, so the run is refused before any device work
    from sc_gb300._lib import ScError

    c = next(c for c in CASES if c["name"] == "o7_contact")
    inp = c["inputs"]
    top = inp["top.init"].replace("S: {\nparticles: 2\n}", "S: {\nparticles: 2\nparticles: 2\nbond1: 50 1.0\n}")
    top = top.replace("S 100", "S 50")
    assert top != inp["top.init"]
    opts = _sub(_sub(_sub(inp["options"], "chainprob", "0.1"), "chainmmx", "0.3"), "chainrmx", "10")
    s = System.from_text(opts, top, inp["config.init"])
    s.wl_load(text=inp["wl.dat"])
    assert s.wl_info().currorder[0] == c["ref"]["currorder"][0]
    with pytest.raises(ScError) as e:
        s.simulate(nsweeps=1)
    assert e.value.code == ERR_UNSUPPORTED and "order 7" in str(e.value)
    s.close()
