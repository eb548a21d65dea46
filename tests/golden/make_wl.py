#!/usr/bin/env python3
"""Golden vectors of the Wang-Landau tests (tests/golden/wl/cases.json.gz).

Runs the reference itself, compiled from its own sources by ``oracle/Makefile``
(``make -C oracle ref``), on seeded synthetic systems written by this script, each with
a weights file ``wl.dat``:

* ``oracle/_ref/ref_dump`` (the reference's ``WangLandau::init`` and ``write``): the
  starting bins, the system centre and sysvolume, and the text the reference writes back
  for the weights it read;
* ``oracle/_ref/sc_ref`` (the reference's own ``main``), several seeds: adaptive runs of
  the two-particle distance case and fixed-weight runs of the orientation, system-centre,
  contact-count and mesh-hole cases, the weights and histogram they end with
  (``wl-new.dat``), for the comparisons.

Run here (needs the reference tree):  python tests/golden/make_wl.py
"""
import gzip
import json
import math
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import config_text, options_text, rand_perp, rand_unit, top_text  # noqa: E402

REPO = os.path.dirname(os.path.dirname(HERE))
# the reference checkout, as the oracle's recipe locates it (SC_REFERENCE overrides)
from make_golden import REF_ROOT  # noqa: E402

MEMBRANE = os.path.join(REF_ROOT, "Tests", "SC_PSC_MEMBRANE_WANG")
DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")
SCREF = os.path.join(REPO, "oracle", "_ref", "sc_ref")


def wl_text(alpha, orders, weights, hists=None):
    """orders: list of tuples (one or two order values per bin, order 0 fastest)."""
    s = "%.17g\n" % alpha
    for k, o in enumerate(orders):
        h = 0 if hists is None else hists[k]
        s += " ".join("%.17g" % v for v in o) + " %.17g %d\n" % (weights[k], h)
    return s


def grid1(lo, d, n):
    return [(lo + i * d,) for i in range(n)]


def grid2(lo0, d0, n0, lo1, d1, n1):
    return [(lo0 + i * d0, lo1 + j * d1) for j in range(n1) for i in range(n0)]


def bath(rng, box, n, first, min_dist=1.05, first_dist=1.05):
    """n sphere centres (box fractions), at least min_dist apart and first_dist from the
    given centres (real space)."""
    out = []
    for _ in range(200000):
        if len(out) == n:
            return out
        p = rng.random(3)
        ok = True
        for q, lim in [(q, first_dist) for q in first] + [(q, min_dist) for q in out]:
            d = (p - q) * box
            d -= box * np.round(d / box)
            if np.dot(d, d) < lim * lim:
                ok = False
                break
        if ok:
            out.append(p)
    raise RuntimeError("bath: no room for the particles")


def cases():
    rng = np.random.default_rng(20261204)
    out = []
    spn = lambda num, name: (name, num, "SPN", [1.0, 1.0])
    # (1) order 4, xy distance of two spheres that see only each other (type 1 excluded
    # from the bath, type 2); adaptive weights
    box = np.array([6.0, 6.0, 6.0])
    p01 = [np.array([0.2, 0.3, 0.4]), np.array([0.55, 0.5, 0.6])]
    pos = p01 + bath(rng, box, 40, p01)
    dirs = rand_unit(rng, len(pos))
    top = top_text([spn(1, "A"), spn(2, "B")], [("A", [1], []), ("B", [2], [])], [("A", 2), ("B", 40)])
    top += "[EXCLUDE]\n1 2\n"
    out.append(dict(name="o4_pair", wlm=(4, 0), options=dict(wlm="4 0", transmx=0.3, rotmx=0.0, nsweeps=60000,
                                                               seed=11, shave=0, ptype=0),
                    top=top, config=config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs)),
                    wl=wl_text(0.5, grid1(0.1, 0.1, 43), [0.0] * 43)))
    # (2) order 3, z component of a free spherocylinder's axis, fixed linear bias
    box = np.array([6.0, 6.0, 6.0])
    p0 = [np.array([0.5, 0.5, 0.5])]
    pos = p0 + bath(rng, box, 40, p0, first_dist=2.1)
    dirs = rand_unit(rng, len(pos))
    psc = ("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 2.0, 0.0])
    top = top_text([psc, spn(2, "B")], [("P", [1], []), ("B", [2], [])], [("P", 1), ("B", 40)])
    top += "[EXCLUDE]\n1 2\n"
    orders = grid1(-1.0, 0.05, 41)
    out.append(dict(name="o3_orient", wlm=(3, 0), options=dict(wlm="3 0", transmx=0.2, rotmx=120.0, nsweeps=0,
                                                                 seed=12, shave=0, ptype=0),
                    top=top, config=config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs)),
                    wl=wl_text(1e-12, orders, [1.5 * o[0] for o in orders])))
    # (3) orders 1 and 3 together, as the reference's membrane example (two dimensions)
    box = np.array([6.0, 6.0, 10.0])
    p0 = [np.array([0.5, 0.5, 0.62])]
    pos = p0 + bath(rng, box, 60, p0, first_dist=2.6)
    dirs = rand_unit(rng, len(pos))
    cpsc = ("C", 1, "CPSC", [1.0, 1.0, 1.12, 0.2, 120.0, 10.0, 3.0, 0.0])
    top = top_text([cpsc, ("S", 2, "SPA", [1.0, 1.0, 1.1225, 0.3775])], [("C", [1], []), ("S", [2], [])],
                   [("C", 1), ("S", 60)])
    orders = grid2(-8.0, 0.25, 65, -1.0, 0.1, 21)
    w = [0.01 * k for k in range(len(orders))]
    h = [k % 7 for k in range(len(orders))]
    out.append(dict(name="o1_o3", wlm=(1, 3), options=dict(wlm="1 3", wlmtype=1, transmx=0.2, rotmx=20.0, nsweeps=0,
                                                             seed=13, shave=0, ptype=0),
                    top=top, config=config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs)),
                    wl=wl_text(0.25, orders, w, h)))
    # (4) box lengths x and y (two dimensions)
    box = np.array([7.0, 7.5, 8.0])
    pos = bath(rng, box, 30, [])
    dirs = rand_unit(rng, len(pos))
    top = top_text([spn(1, "A")], [("A", [1], [])], [("A", 30)])
    orders = grid2(6.0, 0.1, 21, 6.0, 0.1, 31)
    out.append(dict(name="o8_o9", wlm=(8, 9), options=dict(wlm="8 9", transmx=0.2, rotmx=0.0, nsweeps=0, seed=14,
                                                             shave=1, ptype=0, edge_mx=0.1),
                    top=top, config=config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs)),
                    wl=wl_text(0.1, orders, [math.sin(0.1 * k) for k in range(len(orders))])))
    # (5) order 1 alone, a bath that interacts (one dimension), and order 9 alone
    box = np.array([6.5, 6.5, 9.0])
    p0 = [np.array([0.3, 0.7, 0.2])]
    pos = p0 + bath(rng, box, 50, p0)
    dirs = rand_unit(rng, len(pos))
    top = top_text([spn(1, "A"), ("S", 2, "SPA", [1.0, 1.0, 1.1225, 0.3775])], [("A", [1], []), ("S", [2], [])],
                   [("A", 1), ("S", 50)])
    cfg = config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs))
    out.append(dict(name="o1_bath", wlm=(1, 0), options=dict(wlm="1 0", transmx=0.2, rotmx=0.0, nsweeps=0, seed=15,
                                                               shave=0, ptype=0),
                    top=top, config=cfg, wl=wl_text(0.125, grid1(-4.5, 0.1, 91), [0.0] * 91)))
    out.append(dict(name="o9_box", wlm=(9, 0), options=dict(wlm="9 0", transmx=0.2, rotmx=0.0, nsweeps=0, seed=16,
                                                              shave=1, ptype=5, edge_mx=0.1),
                    top=top, config=cfg, wl=wl_text(0.0, grid1(6.0, 0.05, 21), [0.2 * k for k in range(21)])))
    # (6) a weight wall on the box length in y (ptype 5): weights 0 inside bins 5..15, -1e4
    # outside, fixed (alpha 0)
    wall = [0.0 if 5 <= k <= 15 else -1e4 for k in range(21)]
    out.append(dict(name="o9_wall", wlm=(9, 0), options=dict(wlm="9 0", transmx=0.2, rotmx=0.0, nsweeps=3000,
                                                               seed=17, shave=1, ptype=5, edge_mx=0.1),
                    top=top, config=cfg, wl=wl_text(0.0, grid1(6.0, 0.05, 21), wall)))
    # (8) order 1 under fixed weights (alpha 0): a harmonic well w = -0.5 z^2 for the height
    # of particle 0 above the system centre, in the interacting bath of (5); the reference's
    # histograms of several seeds bound the effect of the centre's unbiased moves
    zs = grid1(-4.5, 0.1, 91)
    out.append(dict(name="o1_fixed", wlm=(1, 0), options=dict(wlm="1 0", transmx=0.2, rotmx=0.0, nsweeps=20000,
                                                                seed=18, shave=0, ptype=0),
                    top=top, config=cfg, wl=wl_text(0.0, zs, [-0.5 * z[0] * z[0] for z in zs])))
    # (9) order 7, the number of bath spheres (type 2, wlmtype) within 6 sigma of particle 0,
    # under fixed weights linear in the count (alpha 0); NVT, then NPT (isotropic volume moves
    # recount the contacts in the trial box)
    box = np.array([12.0, 12.0, 12.0])
    p0 = [np.array([0.5, 0.5, 0.5])]
    pos = p0 + bath(rng, box, 100, p0)
    dirs = rand_unit(rng, len(pos))
    top = top_text([spn(1, "A"), ("S", 2, "SPA", [1.0, 1.0, 1.1225, 0.3775])], [("A", [1], []), ("S", [2], [])],
                   [("A", 1), ("S", 100)])
    cfg = config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs))
    counts = grid1(0.0, 1.0, 101)
    wl7 = wl_text(0.0, counts, [0.08 * c[0] for c in counts])
    out.append(dict(name="o7_contact", wlm=(7, 0), options=dict(wlm="7 0", wlmtype=2, transmx=0.5, rotmx=0.0,
                                                                  nsweeps=4000, seed=19, shave=0, ptype=0),
                    top=top, config=cfg, wl=wl7))
    out.append(dict(name="o7_npt", wlm=(7, 0), options=dict(wlm="7 0", wlmtype=2, transmx=0.5, rotmx=0.0,
                                                              nsweeps=4000, seed=20, shave=1, ptype=1, press=0.06,
                                                              edge_mx=0.2),
                    top=top, config=cfg, wl=wl7))
    # (10) order 2, the largest hole of the xy mesh (squares sigma / 3) that 60 spheres of type
    # 2 (wlmtype) leave, under fixed weights linear in its bin (alpha 0)
    box = np.array([8.0, 8.0, 8.0])
    p0 = [np.array([0.5, 0.5, 0.5])]
    pos = p0 + bath(rng, box, 60, p0)
    dirs = rand_unit(rng, len(pos))
    top = top_text([spn(1, "A"), spn(2, "B")], [("A", [1], []), ("B", [2], [])], [("A", 1), ("B", 60)])
    holes = grid1(0.0, 4.0, 145)
    out.append(dict(name="o2_mesh", wlm=(2, 0), options=dict(wlm="2 0", wlmtype=2, transmx=0.4, rotmx=0.0,
                                                               nsweeps=6000, seed=21, shave=0, ptype=0),
                    top=top, config=config_text(box, np.array(pos) * box, dirs, rand_perp(rng, dirs)),
                    wl=wl_text(0.0, holes, [0.05 * k for k in range(len(holes))])))
    # (7) the reference's own membrane test (Tests/SC_PSC_MEMBRANE_WANG/scOOP_test): a CPSC
    # protein and 200 three-bead lipids, orders 1 and 3, NPT (ptype 2) with chain moves, and
    # the converged weights of its legacy run (wl_orig_results.dat) as the weights file.  Its
    # options file lacks the ptype and press lines, which the reference requires (sim.h:177);
    # they are taken from the test's other options file (ptype 2, press 0).
    if os.path.isdir(MEMBRANE):
        d = os.path.join(MEMBRANE, "scOOP_test")
        opts = open(os.path.join(d, "options")).read().rstrip("\n") + "\nptype = 2\npress = 0.0\n"
        out.append(dict(name="membrane_ref", wlm=(1, 3), options_text=opts,
                        top=open(os.path.join(d, "top.init")).read(),
                        config=open(os.path.join(d, "config.init")).read(),
                        wl=open(os.path.join(d, "wl_orig_results.dat")).read()))
    return out


def case_options(c):
    return c["options_text"] if "options_text" in c else options_text(**c["options"])


def write_case(d, c):
    with open(os.path.join(d, "options"), "w") as f:
        f.write(case_options(c))
    with open(os.path.join(d, "top.init"), "w") as f:
        f.write(c["top"])
    with open(os.path.join(d, "config.init"), "w") as f:
        f.write(c["config"])
    with open(os.path.join(d, "wl.dat"), "w") as f:
        f.write(c["wl"])


def read_wl(path):
    rows = []
    alpha = None
    for line in open(path):
        t = line.split()
        if not t:
            continue
        if alpha is None:
            alpha = float(t[0])
        else:
            rows.append([float(x) for x in t])
    return alpha, rows


def main():
    for exe in (DUMP, SCREF):
        if not os.path.exists(exe):
            sys.exit(f"{exe} missing: run make -C oracle ref first")
    only = sys.argv[1:]           # names: regenerate those cases only, keep the others
    old = []
    path = os.path.join(HERE, "wl", "cases.json.gz")
    if only and os.path.exists(path):
        with gzip.open(path, "rt") as f:
            old = [e for e in json.load(f)["cases"] if e["name"] not in only]
    result = []
    for c in cases():
        if only and c["name"] not in only:
            continue
        tmp = tempfile.mkdtemp()
        try:
            write_case(tmp, c)
            r = subprocess.run([DUMP, tmp, "0", "0"], capture_output=True, text=True, check=True)
            dump = json.loads(r.stdout)
            entry = {"name": c["name"], "inputs": {"options": case_options(c), "top.init": c["top"],
                                                   "config.init": c["config"], "wl.dat": c["wl"]},
                     "ref": dump["wl"], "n": dump["n"],
                     "system": {k: dump[k] for k in ("box", "sqmaxcut", "ia_params", "particles", "molecules")}}
            if c["name"] in ("o4_pair", "o3_orient", "o9_wall", "o1_fixed", "o7_contact", "o7_npt", "o2_mesh"):
                # the reference's own adaptive runs, three seeds
                runs = []
                six = (101, 202, 303, 404, 505, 606)
                twelve = six + (707, 808, 909, 1010, 1111, 1212)
                seeds = {"o9_wall": (101,), "o1_fixed": six, "o7_contact": six, "o7_npt": twelve,
                         "o2_mesh": six}.get(c["name"], (101, 202, 303))
                for seed in seeds:
                    opts = dict(c["options"], seed=seed)
                    if c["name"] == "o3_orient":
                        opts["nsweeps"] = 20000
                    with open(os.path.join(tmp, "options"), "w") as f:
                        f.write(options_text(**opts))
                    with open(os.path.join(tmp, "wl.dat"), "w") as f:
                        f.write(c["wl"])
                    subprocess.run([SCREF], cwd=tmp, capture_output=True, text=True, check=True, timeout=1800)
                    alpha, rows = read_wl(os.path.join(tmp, "wl-new.dat"))
                    runs.append({"seed": seed, "alpha": alpha, "weights": [r[1] for r in rows],
                                 "hist": [int(r[2]) for r in rows]})
                entry["ref_runs"] = runs
            result.append(entry)
            print(c["name"], dump["wl"]["currorder"], flush=True)
        finally:
            shutil.rmtree(tmp)
    os.makedirs(os.path.join(HERE, "wl"), exist_ok=True)
    order = [c["name"] for c in cases()]
    result = sorted(old + result, key=lambda e: order.index(e["name"]) if e["name"] in order else len(order))
    with gzip.open(path, "wt") as f:
        json.dump({"generator": "tests/golden/make_wl.py", "cases": result}, f)


if __name__ == "__main__":
    main()
