#!/usr/bin/env python3
"""Ensemble goldens: averages sampled by the reference's own Metropolis loop.

Runs the reference binary built from its own sources (oracle/_ref/sc_ref, see
oracle/Makefile) on seeded synthetic systems, several independent seeds each, and
stores the time series it writes (energy.dat: total energy and alignmentOrder;
stat.dat: volume) as tests/golden/ens_<name>.json together with the inputs.  The
GPU sampler must reproduce the averages within 2 standard errors.

Run here (needs the reference tree): python tests/golden/make_ensemble.py
"""
import json
import math
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from make_golden import OPTION_KEYS, config_text, rand_perp, rand_unit, top_text  # noqa: E402

SC_REF = os.path.join(REPO, "oracle", "_ref", "sc_ref")


def seg_dist(p1, d1, p2, d2, L):
    """Closest distance of two segments of length L (numpy, for initial placement only)."""
    best = 1e9
    for s in np.linspace(-L / 2, L / 2, 9):
        a = p1 + s * d1
        t = np.clip(np.dot(a - p2, d2), -L / 2, L / 2)
        best = min(best, np.linalg.norm(a - (p2 + t * d2)))
    return best


def place(rng, n, box, L, dmin=1.05, types=None):
    pos, dirs = [], []
    tries = 0
    while len(pos) < n:
        tries += 1
        p = rng.uniform(0, 1, 3) * box
        d = rand_unit(rng, 1)[0]
        ok = True
        for q, e in zip(pos, dirs):
            r = p - q
            r -= box * np.round(r / box)
            if np.linalg.norm(r) > L + dmin:
                continue
            if seg_dist(q + r, d, q, e, L) < dmin:
                ok = False
                break
        if ok:
            pos.append(p)
            dirs.append(d)
    pos, dirs = np.array(pos), np.array(dirs)
    return pos, dirs, rand_perp(rng, dirs)


def cases():
    rng = np.random.default_rng(31337)
    out = {}
    # PSC, the benchmark model, NVT
    n = 250
    phi = 0.2
    L = 3.0
    box = np.full(3, (n * (math.pi / 6 + math.pi / 4 * L) / phi) ** (1 / 3))
    pos, dirs, pds = place(rng, n, box, L)
    out["psc_nvt"] = dict(
        top=top_text([("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0])], [("P", [1], [])], [("P", n)]),
        config=config_text(box, pos, dirs, pds),
        opts=dict(temper=0.6, transmx=0.35, rotmx=30.0, pairlist_update=10),
        nsweeps=24000, report=20, seeds=6, burn=4000)
    # CPSC + SPA mixture, NPT
    n = 200
    box = np.full(3, 14.5)
    pos, dirs, pds = place(rng, n, box, L)
    out["cpsc_spa_npt"] = dict(
        top=top_text([("C", 1, "CPSC", [1.0, 1.0, 1.12, 0.2, 120.0, 10.0, L, 0.0]),
                      ("A", 2, "SPA", [0.5, 1.0, 1.1225, 0.3775])],
                     [("C", [1], []), ("A", [2], [])], [("C", 100), ("A", 100)]),
        config=config_text(box, pos, dirs, pds),
        opts=dict(temper=1.0, press=0.5, ptype=1, shave=1, edge_mx=0.25, transmx=0.35, rotmx=30.0,
                  pairlist_update=0),
        nsweeps=16000, report=20, seeds=6, burn=4000)
    # three-bead lipids (SPN head, two TPSC tails, bond1), chain + single-particle moves, NVT
    sys.path.insert(0, REPO)
    from sc_gb300 import workloads

    opts_text, top, config = workloads.lipids_dilute(64, seed=3)
    lip_opts = dict(l.split(" = ") for l in opts_text.strip().splitlines())
    out["lipids_chain"] = dict(
        top=top, config=config, n_particles=192,
        opts=dict(temper=1.5, transmx=0.3, rotmx=20.0, chainprob=0.2, chainmmx=0.3, chainrmx=15.0,
                  pairlist_update=10),
        nsweeps=30000, report=20, seeds=6, burn=5000)
    assert float(lip_opts["chainprob"]) == 0.2
    # the benchmark's own state points: 1000 PSC at packing fraction 0.1, T = 1 (NVT), and the
    # CPSC + SPA mixture at P* = 0.5, T = 1 (NPT, isotropic volume moves), reduced to 500
    # particles; the nematic order S2 from the reference's own movie frames
    # the first case with axial rotations (partAxialRotate: rotation axes in a cone of 40 degrees
    # around the particle axis), S2 and the alignment order
    out["psc_cone"] = dict(out["psc_nvt"], opts=dict(out["psc_nvt"]["opts"], coneAngle=40.0), s2=True, pre=20000,
                           burn=2000)
    # Both start from one configuration the reference itself has equilibrated (`pre` sweeps from
    # the seeded start): the patchy particles keep aggregating slowly from a random start, and
    # averages over a relaxing window would depend on each sampler's kinetics.
    for name, texts, pre, nsw, burn in (("psc_c0", workloads.nvt_psc(1000, phi=0.1, seed=1), 30000, 8000, 1000),
                                        ("mixture_c1", workloads.npt_cpsc_spa(500, phi=0.1, seed=1), 60000, 12000,
                                         2000)):
        opts_text, top, config = texts
        base = dict(l.split(" = ") for l in opts_text.strip().splitlines())
        base.update(pairlist_update="10", nequil="0")
        out[name] = dict(top=top, config=config, opts=base, nsweeps=nsw, report=20, seeds=6, burn=burn, s2=True,
                         pre=pre)
    # grand-canonical (muVT) moves, one every sweep (nGrandCanon = 1): attractive spheres as the
    # only species, and patchy spherocylinders inserted and removed among fixed spheres (the
    # species listed last, so removals inside its block shift the particles behind); the count
    # from the reference's movie frames, the total energy from energy.dat
    box = np.full(3, 8.0)
    pos = place_spheres(rng, 30, box, 1.1)
    out["gc_spa"] = dict(
        top=top_text([("A", 1, "SPA", [1.0, 1.0, 1.1225, 0.5])], [("A", [1], ["ACTIVITY: 0.1"])], [("A", 30)]),
        config=config_text(box, pos, rand_unit(rng, 30), rand_perp(rng, rand_unit(rng, 30))),
        opts=dict(temper=1.0, transmx=0.6, rotmx=30.0, nGrandCanon=1, pairlist_update=0),
        nsweeps=24000, report=20, seeds=32, burn=4000, gc=True)
    box = np.full(3, 12.0)
    ps, ds, qs = place(rng, 15, box, L)
    sp = []
    while len(sp) < 20:          # spheres clear of the spherocylinders and of each other
        p = rng.uniform(0, 1, 3) * box
        if all(np.linalg.norm((p - q) - box * np.round((p - q) / box)) > 1.2 for q in sp) and all(
                seg_dist(p, np.array([0.0, 0.0, 1.0]), p + ((q - p) - box * np.round((q - p) / box)), d, L) > 1.2
                and np.linalg.norm((p - q) - box * np.round((p - q) / box)) > 0 for q, d in zip(ps, ds)):
            sp.append(p)
    sp = np.array(sp)
    out["gc_psc"] = dict(
        top=top_text([("A", 2, "SPA", [0.5, 1.0, 1.1225, 0.3775]),
                      ("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0])],
                     [("A", [2], []), ("P", [1], ["ACTIVITY: 0.02"])], [("A", 20), ("P", 15)]),
        config=config_text(box, np.vstack([sp, ps]), np.vstack([rand_unit(rng, 20), ds]),
                           np.vstack([rand_perp(rng, rand_unit(rng, 20)), qs])),
        opts=dict(temper=1.0, transmx=0.5, rotmx=30.0, nGrandCanon=1, pairlist_update=0),
        nsweeps=24000, report=20, seeds=48, burn=4000, gc=True)
    # type switching (switchTypeMove): PSC particles that switch to a CPSC type and back with a
    # chemical-potential difference of 1.6 (read as the int 1 by the reference), beside fixed
    # spheres; the switched fraction from the movie frames' switched column
    box = np.full(3, 16.0)
    ps, ds, qs = place(rng, 150, box, L)
    sp = []
    while len(sp) < 50:
        p = rng.uniform(0, 1, 3) * box
        if all(np.linalg.norm((p - q) - box * np.round((p - q) / box)) > 1.2 for q in sp) and all(
                seg_dist(p, np.array([0.0, 0.0, 1.0]), p + ((q - p) - box * np.round((q - p) / box)), d, L) > 1.2
                for q, d in zip(ps, ds)):
            sp.append(p)
    sp = np.array(sp)
    out["switch_psc"] = dict(
        top=top_text([("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0]),
                      ("Q", 2, "CPSC", [1.0, 1.0, 1.12, 0.2, 120.0, 10.0, L, 0.0]),
                      ("A", 3, "SPA", [0.5, 1.0, 1.1225, 0.3775])],
                     [("P", ["1 2 1.6"], []), ("A", [3], [])], [("P", 150), ("A", 50)]),
        config=config_text(box, np.vstack([ps, sp]), np.vstack([ds, rand_unit(rng, 50)]),
                           np.vstack([qs, rand_perp(rng, rand_unit(rng, 50))])),
        opts=dict(temper=1.0, transmx=0.35, rotmx=30.0, switchprob=0.1, pairlist_update=0),
        nsweeps=24000, report=20, seeds=12, burn=3000, switch_rows=150)
    # every volume coupling of pressureMove (movecreator.cpp:349-546) on one small fluid of
    # attractive spheres (T = 2, P* = 1): ptype 0 one edge at a time, 2 x and y with z kept,
    # 3 x and y with z re-derived to keep the volume (no volume term: the box x from the movie
    # frames is the observable), 4 x alone (the reference's x-or-y test always takes x), 5 y alone
    n = 64
    box = np.full(3, 5.04)
    pos = place_spheres(rng, n, box, 1.0)
    sph = dict(top=top_text([("A", 1, "SPA", [1.0, 1.0, 1.1225, 0.5])], [("A", [1], [])], [("A", n)]),
               config=config_text(box, pos, rand_unit(rng, n), rand_perp(rng, rand_unit(rng, n))),
               nsweeps=20000, report=20, seeds=8, burn=2000)
    for pt in (0, 2, 3, 4, 5):
        out[f"spa_ptype{pt}"] = dict(sph, opts=dict(temper=2.0, press=1.0, ptype=pt, shave=1, edge_mx=0.1,
                                                     transmx=0.25, rotmx=30.0, pairlist_update=10),
                                     box_x=pt == 3)
    return out


def place_spheres(rng, n, box, dmin):
    pos = []
    while len(pos) < n:
        p = rng.uniform(0, 1, 3) * box
        if all(np.linalg.norm((p - q) - box * np.round((p - q) / box)) > dmin for q in pos):
            pos.append(p)
    return np.array(pos)


def pre_equilibrate(c, seed=999):
    """config.last of one reference run of c["pre"] sweeps from c's start (its box and lines,
    which the config.init reader takes as they are)."""
    with tempfile.TemporaryDirectory() as tmp:
        opts = dict(OPTION_KEYS)
        opts.update(c["opts"])
        opts.update(nsweeps=c["pre"], report=c["pre"], seed=seed, paraltemper=opts["temper"], movie=0)
        with open(os.path.join(tmp, "options"), "w") as f:
            f.write("".join(f"{k} = {v}\n" for k, v in opts.items()))
        with open(os.path.join(tmp, "top.init"), "w") as f:
            f.write(c["top"])
        with open(os.path.join(tmp, "config.init"), "w") as f:
            f.write(c["config"])
        subprocess.run([SC_REF], cwd=tmp, check=True, capture_output=True)
        return open(os.path.join(tmp, "config.last")).read()


def nematic_s2(dirs):
    """Largest eigenvalue of <3/2 u u^T - 1/2 I> over unit axes (rows of dirs)."""
    q = 1.5 * (dirs.T @ dirs) / len(dirs) - 0.5 * np.eye(3)
    return float(np.linalg.eigvalsh(q)[-1])


def movie_s2(path, sc_rows):
    """S2 of every frame of the reference's movie file (frames: count line, 'sweep S; box ...'
    line, then one 'x y z dx dy dz px py pz switched molType' line per particle)."""
    lines = open(path).read().splitlines()
    out, k = [], 0
    while k < len(lines):
        n = int(lines[k].split()[0])
        sweep = int(lines[k + 1].split(";")[0].split()[1])
        rows = lines[k + 2: k + 2 + n]
        dirs = np.array([[float(x) for x in r.split()[3:6]] for r in rows])[sc_rows]
        out.append((sweep, nematic_s2(dirs)))
        k += 2 + n
    return out


def run_one(c, seed):
    with tempfile.TemporaryDirectory() as tmp:
        opts = dict(OPTION_KEYS)
        opts.update(c["opts"])
        opts.update(nsweeps=c["nsweeps"], report=c["report"], seed=seed, paraltemper=opts["temper"])
        if c.get("s2") or c.get("gc") or c.get("switch_rows") or c.get("box_x"):
            opts.update(movie=c["report"])
        with open(os.path.join(tmp, "options"), "w") as f:
            f.write("".join(f"{k} = {v}\n" for k, v in opts.items()))
        with open(os.path.join(tmp, "top.init"), "w") as f:
            f.write(c["top"])
        with open(os.path.join(tmp, "config.init"), "w") as f:
            f.write(c["config"])
        subprocess.run([SC_REF], cwd=tmp, check=True, capture_output=True)
        e, al, vol = [], [], []
        for line in open(os.path.join(tmp, "energy.dat")):
            if line.startswith("#"):
                continue
            sw, rest = line.split(";")
            a, b = rest.split()
            e.append((int(sw), float(a), float(b)))
        for line in open(os.path.join(tmp, "stat.dat")):
            if line.startswith("#"):
                continue
            sw, v = line.split(";")
            vol.append((int(sw), float(v)))
        s2, counts = [], []
        if c.get("s2"):
            n_sc = int(c["top"].split("[System]")[1].split()[1])     # the first [System] entry: the SCs
            s2 = movie_s2(os.path.join(tmp, "movie"), slice(0, n_sc))
        if c.get("gc"):
            counts = movie_counts(os.path.join(tmp, "movie"))
        switched = []
        if c.get("switch_rows"):
            switched = movie_switched(os.path.join(tmp, "movie"), c["switch_rows"])
        box_x = movie_box_x(os.path.join(tmp, "movie")) if c.get("box_x") else []
        return dict(seed=seed, energy=e, volume=vol, s2=s2, counts=counts, switched=switched, box_x=box_x)


def movie_box_x(path):
    """(sweep, box x) of every frame of the reference's movie file ('sweep S; box x y z')."""
    lines = open(path).read().splitlines()
    out, k = [], 0
    while k < len(lines):
        n = int(lines[k].split()[0])
        head = lines[k + 1]
        out.append((int(head.split(";")[0].split()[1]), float(head.split("box")[1].split()[0])))
        k += 2 + n
    return out


def movie_switched(path, rows):
    """(sweep, fraction of the first `rows` particles marked switched) of every movie frame."""
    lines = open(path).read().splitlines()
    out, k = [], 0
    while k < len(lines):
        n = int(lines[k].split()[0])
        sweep = int(lines[k + 1].split(";")[0].split()[1])
        flags = [int(r.split()[9]) for r in lines[k + 2: k + 2 + rows]]
        out.append((sweep, sum(flags) / rows))
        k += 2 + n
    return out


def movie_counts(path):
    """(sweep, particle count) of every frame of the reference's movie file."""
    lines = open(path).read().splitlines()
    out, k = [], 0
    while k < len(lines):
        n = int(lines[k].split()[0])
        out.append((int(lines[k + 1].split(";")[0].split()[1]), n))
        k += 2 + n
    return out


def block_stats(series_per_seed, burn):
    """Mean and standard error from per-seed means after the burn-in (seeds independent)."""
    means = [np.mean([v for s, v in ser if s > burn]) for ser in series_per_seed]
    m = float(np.mean(means))
    se = float(np.std(means, ddof=1) / math.sqrt(len(means)))
    return m, se


def main():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", "-j8"], check=True, capture_output=True)
    only = sys.argv[1:]
    for name, c in cases().items():
        if only and name not in only:
            continue
        if c.get("pre"):
            c["config"] = pre_equilibrate(c)
        with ThreadPoolExecutor(max_workers=min(8, c["seeds"])) as ex:
            runs = list(ex.map(lambda s: run_one(c, s), [1000 + k for k in range(c["seeds"])]))
        n = c.get("n_particles") or sum(
            cnt for _, cnt in [tuple(l.split()) for l in c["top"].split("[System]\n")[1].splitlines() if l.strip()]
            for cnt in [int(cnt)])
        e_ser = [[(s, en / n) for s, en, _ in r["energy"]] for r in runs]
        a_ser = [[(s, al / n) for s, _, al in r["energy"]] for r in runs]
        v_ser = [[(s, v / n) for s, v in r["volume"]] for r in runs]
        series = [("energy_per_particle", e_ser), ("alignment_per_particle", a_ser), ("volume_per_particle", v_ser)]
        if c.get("gc"):     # the count changes: totals, and the count itself
            series = [("energy_total", [[(s, en) for s, en, _ in r["energy"]] for r in runs]),
                      ("particles", [[(s, float(k)) for s, k in r["counts"]] for r in runs])]
        if c.get("s2"):
            series.append(("nematic_s2", [r["s2"] for r in runs]))
        if c.get("switch_rows"):
            series = series[:1] + [("switched_fraction", [r["switched"] for r in runs])]
        if c.get("box_x"):
            series.append(("box_x", [r["box_x"] for r in runs]))
        stats = {k: block_stats(ser, c["burn"]) for k, ser in series}
        out = dict(name=name, n=n, inputs={"top.init": c["top"], "config.init": c["config"]}, options=c["opts"],
                   nsweeps=c["nsweeps"], report=c["report"], burn=c["burn"], seeds=c["seeds"],
                   stats={k: {"mean": m, "se": s} for k, (m, s) in stats.items()})
        with open(os.path.join(HERE, f"ens_{name}.json"), "w") as f:
            json.dump(out, f, indent=1)
        print(name, json.dumps(out["stats"]))


if __name__ == "__main__":
    main()
