#!/usr/bin/env python3
"""Generate the golden vectors of the parity tests.

Runs the reference itself, compiled from its own sources by ``oracle/Makefile``
(``make -C oracle ref``), on two kinds of inputs and stores what it computes as
``tests/golden/<name>.json.gz``:

* the reference's own regression fixtures (``Tests/test_*/new`` and
  ``Tests/volumeChange/*/new`` of robertvacha/SC), whose three input files are
  kept verbatim inside the golden file so the tests can feed them to the
  product's parsers;
* seeded synthetic systems written by this script: dense mixtures of every
  interaction type, chains with every bond / angle kind, aligned stacks that
  drive the parallel-segment branch, and small versions of the benchmark
  systems.

Each golden file holds the inputs, the derived interaction table, the particles
after ``Conf::partVecInit``, E(i,j) with branch verdicts for every ordered pair
that passes the cutoff prefilter, oneToAll for every particle, allToAll,
mol2others for every chain, scripted trial moves and volume trials.

Run here (needs the reference tree):  python tests/golden/make_golden.py [REF_ROOT]
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
REPO = os.path.dirname(os.path.dirname(HERE))


def _reference_root():
    """The reference checkout: the first argument, else the one oracle/Makefile resolves
    (SC_REFERENCE in the environment overrides the recipe's default)."""
    if len(sys.argv) > 1:
        return sys.argv[1]
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "print-ref"], capture_output=True,
                       text=True, check=True)
    return os.path.dirname(r.stdout.strip())


REF_ROOT = _reference_root()
DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")

OPTION_KEYS = dict(
    ptype=1, press=0.0, paralpress=0.0, shave=0, nequil=0, adjust=0, nsweeps=100, paramfrq=0, report=0,
    nrepchange=0, nGrandCanon=0, nClustMove=0, movie=0, chainprob=0.0, transmx=0.1, rotmx=10.0,
    edge_mx=0.0, chainmmx=0.0, chainrmx=0.0, temper=1.0, paraltemper=1.0, wlm=0, wlmtype=0,
    switchprob=0.0, pairlist_update=0, seed=145658, write_cluster=0)


def options_text(**over):
    d = dict(OPTION_KEYS)
    d.update(over)
    if "paraltemper" not in over:
        d["paraltemper"] = d["temper"]
    return "".join(f"{k} = {v}\n" for k, v in d.items())


def top_text(types, molecules, system):
    """types: list of (name, num, geotype, [params]); molecules: list of
    (name, [type per particle], [extra lines]); system: list of (name, count)."""
    s = "[Types]\n"
    for name, num, geo, par in types:
        s += f"{name} {num} {geo} " + " ".join(repr(float(p)) for p in par) + "\n"
    s += "[Molecules]\n"
    for name, parts, extra in molecules:
        s += f"{name}: {{\n"
        for t in parts:
            s += f"particles: {t}\n"
        for line in extra:
            s += line + "\n"
        s += "}\n"
    s += "[System]\n"
    for name, cnt in system:
        s += f"{name} {cnt}\n"
    return s


def config_text(box, pos, dirs, pds):
    s = "%.17g %.17g %.17g\n" % tuple(box)
    for p, d, q in zip(pos, dirs, pds):
        s += "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g 0\n" % (*p, *d, *q)
    return s


def rand_unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def rand_perp(rng, d):
    v = rand_unit(rng, len(d))
    v -= (v * d).sum(1, keepdims=True) * d
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def chain_config(rng, nmol, size, box, bond=1.0):
    """Chains laid out as loose random walks of roughly the bond length."""
    pos, dirs = [], []
    for _ in range(nmol):
        p = rng.uniform(0, 1, 3) * box
        d = rand_unit(rng, 1)[0]
        for k in range(size):
            pos.append(p.copy())
            dirs.append(d.copy())
            step = rand_unit(rng, 1)[0] * 0.3 + d
            p = p + step / np.linalg.norm(step) * (bond + 2.0)
            d = d + 0.3 * rand_unit(rng, 1)[0]
            d /= np.linalg.norm(d)
    pos = np.array(pos)
    dirs = np.array(dirs)
    return pos, dirs, rand_perp(rng, dirs)


def synthetic_cases():
    cases = {}
    rng = np.random.default_rng(20240601)

    # every interaction type, same SC length (the reference allows only one)
    L = 3.0
    types = [
        ("N", 1, "SCN", [1.0, 1.0, L]),
        ("S", 2, "SCA", [1.0, 1.0, 1.12246205, 0.4, L]),
        ("P", 3, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0]),
        ("C", 4, "CPSC", [1.2, 1.1, 1.23, 0.25, 120.0, 10.0, L, 0.0]),
        ("H", 5, "CHPSC", [1.0, 1.0, 1.12, 0.2, 80.0, 5.0, L, 0.0, 10.0]),
        ("K", 6, "CHCPSC", [0.9, 1.0, 1.15, 0.3, 100.0, 5.0, L, 0.0, -15.0]),
        ("T", 7, "TPSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0, 180.0, 90.0, 10.0]),
        ("U", 8, "TCPSC", [1.0, 1.05, 1.2, 0.2, 70.0, 10.0, L, 0.0, 120.0, 60.0, 5.0]),
        ("V", 9, "TCHPSC", [1.1, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0, 150.0, 90.0, 10.0, 12.0]),
        ("W", 10, "TCHCPSC", [1.0, 1.0, 1.12, 0.2, 100.0, 10.0, L, 0.0, 90.0, 80.0, 5.0, -8.0]),
        ("O", 11, "SPN", [1.0, 0.95]),
        ("A", 12, "SPA", [0.5, 1.0, 1.1225, 0.3775]),
    ]
    per = 16
    n = per * len(types)
    box = np.array([12.5, 12.0, 13.0])
    mols = [(t[0], [t[1]], []) for t in types]
    system = [(t[0], per) for t in types]
    pos = rng.uniform(0, 1, (n, 3)) * box
    dirs = rand_unit(rng, n)
    cases["mix_all_types"] = dict(
        options=options_text(transmx=0.3, rotmx=20.0),
        top=top_text(types, mols, system), config=config_text(box, pos, dirs, rand_perp(rng, dirs)))

    # mixing rules: different sigma / epsilon / pdis / pswitch and parallel factors
    types = [
        ("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 2.0, 0.4]),
        ("Q", 2, "PSC", [1.5, 1.2, 1.35, 0.3, 60.0, 5.0, 2.0, 0.2]),
        ("C", 3, "CPSC", [0.8, 0.9, 1.1, 0.2, 150.0, 10.0, 2.0, -0.3]),
        ("D", 4, "CPSC", [1.0, 1.0, 1.12, 0.2, 120.0, 10.0, 2.0, -0.1]),
        ("A", 5, "SPA", [0.5, 1.0, 1.1225, 0.3775]),
    ]
    per = 30
    n = per * len(types)
    box = np.array([11.0, 11.0, 11.0])
    pos = rng.uniform(0, 1, (n, 3)) * box
    dirs = rand_unit(rng, n)
    cases["mix_params_parallel"] = dict(
        options=options_text(transmx=0.3, rotmx=20.0),
        top=top_text(types, [(t[0], [t[1]], []) for t in types], [(t[0], per) for t in types]),
        config=config_text(box, pos, dirs, rand_perp(rng, dirs)))

    # aligned stacks: identical / antiparallel axes exercise the parallel-segment branch
    types = [("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 3.0, 0.0]),
             ("C", 2, "CPSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 3.0, 0.0])]
    pos, dirs = [], []
    for a in range(6):
        for b in range(6):
            for c in range(4):
                pos.append([1.05 * a + 0.02 * c, 1.1 * b, 3.6 * c + 0.3 * ((a + b) % 3)])
                dirs.append([0.0, 0.0, 1.0 if (a + c) % 2 == 0 else -1.0])
    pos = np.array(pos, float)
    dirs = np.array(dirs, float)
    pds = np.array([[math.cos(0.7 * k), math.sin(0.7 * k), 0.0] for k in range(len(pos))])
    box = np.array([6.3, 6.6, 14.4])
    cases["aligned_stacks"] = dict(
        options=options_text(transmx=0.1, rotmx=5.0),
        top=top_text(types, [("P", [1], []), ("C", [2], [])], [("P", 72), ("C", 72)]),
        config=config_text(box, pos, dirs, pds))

    # chains: bondh + angle1 + angle2 on PSC chains; bondd + bond2 on TCHCPSC chains; SPA-PSC bond1
    types = [("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 2.0, 0.0]),
             ("W", 2, "TCHCPSC", [1.0, 1.0, 1.12, 0.2, 100.0, 10.0, 2.0, 0.0, 90.0, 80.0, 5.0, 10.0]),
             ("A", 3, "SPA", [0.5, 1.0, 1.1225, 0.3775])]
    mols = [("H", [1, 1, 1, 1], ["bondh: 10.0 0.5", "angle1: 5.0 20.0", "angle2: 4.0 30.0"]),
            ("D", [2, 2, 2, 2, 2], ["bondd: 20.0 0.6", "bond2: 3.0 4.5"]),
            ("B", [3, 1, 1], ["bond1: 50.0 1.0", "bond2: 2.0 3.0", "angle1: 3.0 10.0"])]
    p1, d1, q1 = chain_config(rng, 12, 4, np.array([14.0, 14.0, 14.0]))
    p2, d2, q2 = chain_config(rng, 10, 5, np.array([14.0, 14.0, 14.0]))
    p3, d3, q3 = chain_config(rng, 14, 3, np.array([14.0, 14.0, 14.0]))
    cases["chains_bonds_angles"] = dict(
        options=options_text(transmx=0.2, rotmx=10.0, chainprob=0.1),
        top=top_text(types, mols, [("H", 12), ("D", 10), ("B", 14)]),
        config=config_text(np.array([14.0, 14.0, 14.0]), np.vstack([p1, p2, p3]), np.vstack([d1, d2, d3]),
                           np.vstack([q1, q2, q3])))

    # small versions of the benchmark systems
    types = [("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 3.0, 0.0])]
    n = 200
    box = np.full(3, (n * (math.pi / 6 + math.pi / 4 * 3.0) / 0.25) ** (1 / 3))
    pos = rng.uniform(0, 1, (n, 3)) * box
    dirs = rand_unit(rng, n)
    cases["psc_nvt_small"] = dict(options=options_text(transmx=0.3, rotmx=20.0),
                                  top=top_text(types, [("P", [1], [])], [("P", n)]),
                                  config=config_text(box, pos, dirs, rand_perp(rng, dirs)))

    types = [("C", 1, "CPSC", [1.0, 1.0, 1.12, 0.2, 120.0, 10.0, 3.0, 0.0]),
             ("A", 2, "SPA", [0.5, 1.0, 1.1225, 0.3775])]
    n = 300
    box = np.full(3, 12.0)
    pos = rng.uniform(0, 1, (n, 3)) * box
    dirs = rand_unit(rng, n)
    cases["cpsc_spa_npt_small"] = dict(
        options=options_text(transmx=0.3, rotmx=20.0, press=0.5, shave=1, edge_mx=0.2),
        top=top_text(types, [("C", [1], []), ("A", [2], [])], [("C", 150), ("A", 150)]),
        config=config_text(box, pos, dirs, rand_perp(rng, dirs)))

    types = [("H", 1, "SPN", [1.0, 1.0]),
             ("T", 2, "TPSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, 2.0, 0.0, 180.0, 90.0, 10.0])]
    nmol = 60
    box = np.array([12.0, 12.0, 14.0])
    pos, dirs = [], []
    for m in range(nmol):
        layer = m % 2
        x, y = rng.uniform(0, 1, 2) * box[:2]
        zc = box[2] / 2
        sgn = 1.0 if layer == 0 else -1.0
        # head outside, tails pointing to the mid-plane
        pos += [[x, y, zc + sgn * 5.2], [x, y, zc + sgn * 3.6], [x, y, zc + sgn * 1.2]]
        dirs += [[0, 0, 1.0]] * 3
    pos = np.array(pos, float) + rng.normal(scale=0.05, size=(3 * nmol, 3))
    dirs = np.array(dirs, float) + rng.normal(scale=0.1, size=(3 * nmol, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    cases["bilayer_small"] = dict(
        options=options_text(transmx=0.2, rotmx=10.0, chainprob=0.1),
        top=top_text(types, [("L", [1, 2, 2], ["bond1: 50.0 1.0"])], [("L", nmol)]),
        config=config_text(box, pos, dirs, rand_perp(rng, dirs)))

    # switch types ("particles: TYPE SWITCHTYPE DELTA_MU"), and particles that config.init
    # marks switched (they start in their switch type, whose patch vectors Particle::init
    # derives): PSC <-> CPSC, TPSC <-> TCHPSC, and spheres without a switch type
    rng_s = np.random.default_rng(20261204)
    types = [("P", 1, "PSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0]),
             ("C", 2, "CPSC", [1.2, 1.1, 1.23, 0.25, 120.0, 10.0, L, 0.0]),
             ("T", 3, "TPSC", [1.0, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0, 180.0, 90.0, 10.0]),
             ("V", 4, "TCHPSC", [1.1, 1.0, 1.12, 0.2, 90.0, 10.0, L, 0.0, 150.0, 90.0, 10.0, 12.0]),
             ("A", 5, "SPA", [0.8, 1.0, 1.1225, 0.4])]
    counts = [("M", 40), ("N", 30), ("S", 30)]
    n = sum(c for _, c in counts)
    box = np.array([11.0, 11.5, 12.0])
    pos = rng_s.uniform(0, 1, (n, 3)) * box
    dirs = rand_unit(rng_s, n)
    flags = np.concatenate([rng_s.integers(0, 2, 70), np.zeros(30, int)])
    cfg = config_text(box, pos, dirs, rand_perp(rng_s, dirs))
    lines = cfg.splitlines()
    lines = [lines[0]] + [l[:-1] + str(f) for l, f in zip(lines[1:], flags)]    # the switched column
    cases["switched_types"] = dict(
        options=options_text(transmx=0.2, rotmx=10.0, switchprob=0.1),
        top=top_text(types, [("M", ["1 2 0.7"], []), ("N", ["3 4 -1.5"], []), ("S", [5], [])], counts),
        config="\n".join(lines) + "\n")
    return cases


def run_dump(workdir, ntrials=48, max_i=None):
    args = [DUMP, workdir, str(ntrials)] + ([str(max_i)] if max_i else [])
    res = subprocess.run(args, capture_output=True, text=True, check=True)
    return json.loads(res.stdout)


def save(name, inputs, dump, origin):
    out = dict(name=name, origin=origin, inputs=inputs, ref=dump)
    path = os.path.join(HERE, name + ".json.gz")
    with gzip.open(path, "wt", compresslevel=9) as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"{name}: n={dump['n']} pairs={len(dump['pairs'])} -> {os.path.getsize(path) // 1024} KiB")


def main():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={REF_ROOT}/scOOP", "-j8"],
                   check=True, capture_output=True)
    tests = os.path.join(REF_ROOT, "Tests")
    fixtures = sorted(d for d in os.listdir(tests) if d.startswith("test_") and d[5:7].isdigit())
    dirs = [(f"ref_{d}", os.path.join(tests, d, "new"), f"Tests/{d}/new") for d in fixtures]
    dirs += [(f"ref_volumeChange_{v}", os.path.join(tests, "volumeChange", v, "new"), f"Tests/volumeChange/{v}/new")
             for v in sorted(os.listdir(os.path.join(tests, "volumeChange"))) if os.path.isdir(os.path.join(tests, "volumeChange", v))]
    only = sys.argv[2:]          # synthetic case names: regenerate those only
    for name, src, origin in ([] if only else dirs):
        with tempfile.TemporaryDirectory() as tmp:
            inputs = {}
            for fn in ("options", "top.init", "config.init"):
                shutil.copy(os.path.join(src, fn), tmp)
                inputs[fn] = open(os.path.join(src, fn), encoding="latin-1").read()
            save(name, inputs, run_dump(tmp), origin)
    for name, c in synthetic_cases().items():
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            inputs = {"options": c["options"], "top.init": c["top"], "config.init": c["config"]}
            for fn, txt in inputs.items():
                with open(os.path.join(tmp, fn), "w") as f:
                    f.write(txt)
            save("syn_" + name, inputs, run_dump(tmp), "synthetic (tests/golden/make_golden.py)")


if __name__ == "__main__":
    main()
