#!/usr/bin/env python3
"""Benchmark: attempted Metropolis moves per second on one GB300.

Workload (default): the NPT binary mixture -- 4000 particles, 2000 CPSC (length 3,
cylindrical patch 120 deg) + 2000 attractive spheres SPA (sigma 1, eps 0.5 kT, range
1.5), P* = 0.5, T = 1, one isotropic volume move per sweep -- as a seeded synthetic
start (sc_gb300/workloads.py).  A step is one sweep: N attempted single-particle
moves on the checkerboard plus the volume move, all through the C ABI.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed moves/s (CUDA events on the library's
stream, L2 flushed between steps); `e2e` is the same metric through the public API
with host buffers (state uploaded before and downloaded after every step).
`--impl reference` times the CPU restatement of the reference's own loop (oracle/,
sequential Metropolis with the reference's Verlet list and O(N^2) volume move) on
all host cores, independent seeds per core.

Sections of the same line (rank 0, default run): `replicas` (64 uneven parallel-tempering
replicas in one batch against the same replicas one after another), `surrogate` (65,536
PSC/CPSC, plain against delayed acceptance with the network trained in the run),
`bilayer` (30,000-particle lipid bilayers with chain moves), `wang_landau` (a particle
above a bilayer with and without Wang-Landau weights, eight walkers sharing one table,
and the oracle's sequential loop with the bias as the CPU baseline).  `--only <section>`
runs one of them alone.
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "MC moves/s on 1 GB300: plain FP64 kernel vs surrogate delayed-acceptance"
UNIT = "moves/s"
WORKLOAD = "npt_cpsc_spa_4000"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--only", default="all", choices=["all", "main", "replicas", "surrogate", "bilayer", "wl"],
                    help="run one section alone (prints that section's JSON)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(seconds, dist=None, device="cpu"):
    """The slowest rank's time (the whole job's time: ranks run independent replicas, so
    the job's moves/s is the sum of all ranks' moves over this time)."""
    if dist is None:
        return seconds
    import torch

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profiled_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` from the committed ncu summary of this workload
    (profiles/<kernel>_<workload>.md, line 'traffic_bytes_per_launch = N'), else None."""
    import re

    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        with open(path) as f:
            m = re.search(r"traffic_bytes_per_launch\s*=\s*([0-9.eE+]+)", f.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def open_workload(name, seed):
    from sc_gb300 import System, workloads

    opts, top, cfg = workloads.WORKLOADS[name](seed)
    return System.from_text(opts, top, cfg), (opts, top, cfg)


def oracle_system(texts, seed):
    """The oracle's view of the same start: parameters derived by the oracle itself."""
    import numpy as np

    import oracle_ffi as O
    from sc_gb300 import System

    opts, top, cfg = texts
    s = System.from_text(opts, top, cfg)
    parts = s.particles()
    box = list(s.box)
    p = s.default_run()
    s.close()
    types, excl = O.parse_types(top)
    arr = (O.TypeIn * len(types))(*types)
    table = (O.Param * (O.MAXT * O.MAXT))()
    sq, mc = C.c_double(), C.c_double()
    assert O.lib().or_derive_params(arr, len(types), excl.ctypes.data, table, C.byref(sq), C.byref(mc)) == 0
    op = (O.Particle * len(parts))()
    for k, q in enumerate(parts):
        op[k].pos, op[k].dir = O.vec(q.pos), O.vec(q.dir)
        for m in range(2):
            op[k].pd[m], op[k].ch[m] = O.vec(q.patchdir[m]), O.vec(q.chdir[m])
        for m in range(4):
            op[k].ps[m] = O.vec(q.patchsides[m])
        op[k].type, op[k].molType = q.type, q.molType
    nmol = max(q.molType for q in parts) + 1
    mols = (O.MolType * nmol)()
    for m in range(nmol):
        mols[m].size = 1
        for key in ("bond1", "bond2", "bondd", "bondh", "angle1", "angle2"):
            setattr(mols[m], key + "c", -1.0)
    sysm = O.System()
    sysm.n, sysm.nmol = len(parts), nmol
    sysm.p = C.cast(op, C.POINTER(O.Particle))
    sysm.mols = C.cast(mols, C.POINTER(O.MolType))
    sysm.params = C.cast(table, C.POINTER(O.Param))
    for k in range(3):
        sysm.box[k] = box[k]
    sysm.sqmaxcut = sq.value
    o = O.McOpts()
    o.seed = seed
    o.temper, o.press, o.shave = p.temper, p.press, 1.0 if p.volume_every else 0.0
    o.transmx, o.rot_angle, o.edge_mx = p.transmx, p.rot_angle, p.edge_mx
    o.ptype = p.ptype
    o.pairlist_update = 10
    keep = (op, mols, table, arr)
    return sysm, o, len(parts), keep


def _oracle_molecules(top, O):
    """Molecule records of a top.init for the oracle: size, first particle, count and bond
    constants of each [Molecules] entry in definition order (the molType index), placed in
    the particle vector in [System] order (Inicializer::setParticlesParamss)."""
    defs, order, key, cur = [], [], None, None
    for raw in top.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if line.startswith("["):
            key = line[1:].split("]")[0].strip().upper()
            continue
        if key == "MOLECULES":
            if "{" in line:
                cur = {"name": line.split(":")[0].strip(), "size": 0, "bonds": {}}
                defs.append(cur)
            elif line.startswith("}"):
                cur = None
            elif cur is not None and ":" in line:
                k, v = line.split(":", 1)
                k = k.strip().lower()
                if k == "particles":
                    cur["size"] += 1
                else:
                    cur["bonds"][k] = [float(x) for x in v.split()[:2]]
        elif key == "SYSTEM":
            name, cnt = line.split()[:2]
            order.append((name, int(cnt)))
    mols = (O.MolType * max(1, len(defs)))()
    first = 0
    starts = {}
    for name, cnt in order:
        d = next(d for d in defs if d["name"] == name)
        starts.setdefault(name, (first, cnt))
        first += d["size"] * cnt
    for k, d in enumerate(defs):
        m = mols[k]
        m.size = d["size"]
        m.first, m.count = starts.get(d["name"], (0, 0))
        for b in ("bond1", "bond2", "bondd", "bondh", "angle1", "angle2"):
            c, eq = d["bonds"].get(b, [-1.0, -1.0])
            setattr(m, b + "c", c)
            setattr(m, b + "eq", eq)
    return mols, len(defs)


def wl_cpu_baseline(texts, wl_text, seed, max_moves=3000):
    """One core of the oracle's sequential loop with the Wang-Landau bias (or_wl_run, the
    reference's partDisplace / partRotate with WangLandau::run / runRot) on a bounded
    sample of the same system and weights: moves/s."""
    import numpy as np

    import oracle_ffi as O

    opts, top, cfg = texts
    sysm, o, n, keep = oracle_system(texts, seed)
    mols, nmol = _oracle_molecules(top, O)
    sysm.mols, sysm.nmol = C.cast(mols, C.POINTER(O.MolType)), nmol
    rows = [l.split() for l in wl_text.splitlines() if l.strip()]
    alpha, rows = float(rows[0][0]), [[float(x) for x in r] for r in rows[1:]]
    two = len(rows[0]) == 4
    o0 = sorted({r[0] for r in rows})
    o1 = sorted({r[1] for r in rows}) if two else [0.0]
    st = O.WlState()
    wlm = [int(x) for x in next(l for l in opts.splitlines() if l.split("=")[0].strip() == "wlm").split("=")[1].split()]
    st.wlm[0], st.wlm[1] = (wlm + [0])[:2]
    st.len[0], st.len[1] = len(o0), len(o1)
    st.minorder[0], st.minorder[1] = o0[0], o1[0]
    st.dorder[0] = (o0[-1] - o0[0]) / (len(o0) - 1)
    st.dorder[1] = (o1[-1] - o1[0]) / (len(o1) - 1) if two else 0.0
    st.alpha = alpha
    w = np.array([r[-2] for r in rows], dtype=np.float64)
    h = np.array([r[-1] for r in rows], dtype=np.int64)
    st.weights = w.ctypes.data_as(C.POINTER(C.c_double))
    st.hist = h.ctypes.data_as(C.POINTER(C.c_long))
    cur = (C.c_long * 2)()
    cm = (C.c_double * 3)()
    sv = C.c_double()
    if O.lib().or_wl_orders(C.byref(sysm), st.wlm, st.minorder, st.dorder, cur, cm, C.byref(sv)) != 0:
        raise RuntimeError("oracle: order parameters outside its restatement")
    st.cur[0], st.cur[1] = cur[0], cur[1]
    o.nsweeps, o.max_moves = 1 << 30, max_moves
    ms = O.McStats()
    O.lib().or_wl_run(C.byref(sysm), C.byref(o), C.byref(st), C.byref(ms))
    return ms.moves / max(ms.seconds, 1e-12), ms.moves


def cpu_run(texts, seed, nsweeps, max_moves):
    import oracle_ffi as O

    sysm, o, n, keep = oracle_system(texts, seed)
    o.nsweeps = nsweeps
    o.max_moves = max_moves
    st = O.McStats()
    O.lib().or_mc_run(C.byref(sysm), C.byref(o), C.byref(st))
    return st.moves, st.seconds


def _worker(args):
    texts, seed, nsweeps, max_moves = args
    return cpu_run(texts, seed, nsweeps, max_moves)


def run_reference(a, rank, world):
    """CPU arm: the oracle's restatement of the reference loop on all host cores."""
    if rank != 0:
        return
    import multiprocessing as mp

    from sc_gb300 import workloads

    texts = workloads.WORKLOADS[a.workload](a.seed)
    n = texts[2].count("\n") - 1
    cores = os.cpu_count() or 1
    # size one step so that warm-up + steps stay within a few minutes
    probe_moves, probe_s = cpu_run(texts, a.seed, 1, n)
    per_move = probe_s / max(1, probe_moves)
    budget = 150.0 / max(1, a.steps + a.warmup)
    step_moves = int(max(100, min(n, budget / per_move)))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_worker, [(texts, a.seed + 100 + k, 1, step_moves * a.warmup) for k in range(cores)])
        t0 = time.perf_counter()
        res = pool.map(_worker, [(texts, a.seed + 1000 + k, 1, step_moves * a.steps) for k in range(cores)])
        wall = time.perf_counter() - t0
    moves = sum(m for m, _ in res)
    value = moves / wall
    sample = (f"{cores} independent seeds x {step_moves * a.steps} moves of {a.workload} (sequential Metropolis, "
              f"reference Verlet list every 10 sweeps, O(N^2) volume move with probability 1/N per move)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * wall / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": a.workload, "n_particles": n, "seed": a.seed, "cores": cores},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_replicas(steps, seed=1):
    """64 parallel-tempering replicas of the PSC model (8 systems of uneven N and density,
    each over a geometric 0.8-1.6 ladder), moved together, exchanges every 100 sweeps;
    against the same 64 replicas run one after another by the single-system loop."""
    from sc_gb300 import ReplicaSet, System, workloads

    systems, temps = workloads.pt_ladders(seed=seed)
    ctxs, T, lad = [], [], []
    for g, texts in enumerate(systems):
        for t in temps:
            ctxs.append(System.from_text(*texts))
            T.append(t)
            lad.append(g)
    R = ReplicaSet(ctxs, T, ladder=lad)
    # the tuner: cell reach (tile size) and kernel variant (colour-phase launches or one
    # dataflow launch per sweep) that move the batch fastest
    best = None
    for s, v in ((1, 0), (2, 0), (1, 4), (2, 4)):
        R.run(4, exchange_every=100, seed=seed, stencil=s, variant=v, check_every=0)   # grid, graph capture
        st, *_ = R.run(8, exchange_every=100, seed=seed, stencil=s, variant=v, check_every=0)
        rate = st.moves / st.seconds
        if best is None or rate > best[2]:
            best = (s, v, rate)
    st, Tout, E, tried, acc = R.run(steps, exchange_every=100, seed=seed + 1, stencil=best[0], variant=best[1],
                                    check_every=0)
    batched = st.moves / st.seconds
    # the two forms together: the same batch with a surrogate first stage (trained on the
    # exact pairs of the ladders' configurations) -- delayed-acceptance sweeps
    from sc_gb300 import Surrogate

    sur = Surrogate(ctxs[0], seed=seed, capacity=4_000_000)
    for g in range(len(systems)):
        sur.collect(ctxs[g * len(temps)])
    sur.train(epochs=6, batch=8192, lr=2e-3, warmup_steps=100, seed=seed)
    for c in ctxs:
        c.set_surrogate(sur)
    std, *_ = R.run(steps, exchange_every=100, seed=seed + 3, stencil=best[0], variant=best[1], check_every=0,
                    delayed=1)
    batched_da = std.moves / std.seconds
    for c in ctxs:
        c.set_surrogate(None)
    sur.close()
    # plain: every replica alone through the single-system loop (same tuned stencil, the
    # kernel variant that runs a single system fastest)
    s1 = System.from_text(*systems[0])
    solo = tune_variant(s1, s1.default_run(), 0, stencil=best[0], candidates=(0, 4))
    s1.close()
    moves = secs = 0.0
    for g, texts in enumerate(systems):
        s1 = System.from_text(*texts)
        s1.simulate(nsweeps=2, seed=seed, stencil=best[0], variant=solo, check_every=0)
        one = s1.simulate(nsweeps=3, seed=seed + 2, stencil=best[0], variant=solo, check_every=0)
        moves += one.moves * len(temps)
        secs += one.seconds * len(temps)
        s1.close()
    plain = moves / secs
    R.close()
    particles = sum(c.n for c in ctxs)
    for c in ctxs:
        c.close()
    return {"workload": "pt64_psc_uneven", "replicas": len(ctxs), "particles": particles, "stencil": best[0],
            "kernel_variant": {"batched": best[1], "plain": solo},
            "batched_moves_per_s": batched, "plain_moves_per_s": plain, "speedup": batched / plain,
            "batched_delayed_moves_per_s": batched_da, "speedup_batched_delayed": batched_da / plain,
            "delayed_stage1_decided": std.da_stage1_rejected / max(1, std.moves),
            "exchanges_tried": int(tried.sum()), "exchange_acceptance": float(acc.sum() / max(1, tried.sum())),
            "sweeps": steps}


def tune_variant(s, p, delayed=0, stencil=0, candidates=None):
    """The move-kernel variant that runs s fastest (bit 0: more CTAs per SM instead of the
    lowest latency per move; bit 1: paired passes, plain moves only; bit 2: one dataflow
    launch per sweep instead of one launch per colour)."""
    best = None
    if candidates is None:
        candidates = (0, 1, 4, 5) if delayed else (0, 1, 2, 3, 4, 5)
    for v in candidates:
        s.simulate(p, nsweeps=2, variant=v, delayed=delayed, stencil=stencil)
        st = s.simulate(p, nsweeps=4, variant=v, delayed=delayed, stencil=stencil)
        rate = st.moves / max(st.seconds, 1e-12)
        if best is None or rate > best[1]:
            best = (v, rate)
    p.variant = best[0]
    return best[0]


def bench_surrogate(steps, seed=1, melt=300, snapshots=30, gap=10, epochs=8):
    """Surrogate delayed acceptance on 65,536 PSC/CPSC (50/50, packing fraction 0.2, T=1):
    the aligned start is melted, the exact kernel's pairs of `snapshots` configurations
    train the network (on the GPU), then plain and delayed-acceptance sweeps are timed
    alike (CUDA events, L2 flushed between one-sweep steps)."""
    import torch

    from sc_gb300 import Surrogate, System, workloads

    s = System.from_text(*workloads.psc_cpsc(65536, phi=0.2, seed=seed))
    t0 = time.perf_counter()
    s.simulate(nsweeps=melt, seed=seed, check_every=0)
    melt_s = time.perf_counter() - t0
    sur = Surrogate(s, seed=seed, capacity=12_000_000)
    t0 = time.perf_counter()
    for k in range(snapshots):
        s.simulate(nsweeps=gap, seed=seed + 1 + k, check_every=0)
        sur.collect(s)
    collect_s = time.perf_counter() - t0
    tr, losses = sur.train(epochs=epochs, batch=8192, lr=2e-3, warmup_steps=200, seed=seed)
    s.simulate(nsweeps=gap, seed=seed + 999, check_every=0)
    ev = sur.evaluate(s)                 # a configuration the network was not trained on
    s.set_surrogate(sur)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    run_seed = seed + 4242
    pt = s.default_run()
    pt.seed, pt.check_every = run_seed, 0
    variants = {0: tune_variant(s, pt, 0), 1: tune_variant(s, pt, 1)}   # each mode its fastest kernel

    def timed(delayed):
        variant = variants[delayed]
        s.simulate(nsweeps=3, seed=run_seed, check_every=0, delayed=delayed, variant=variant)
        dev = 0.0
        tot = dict(moves=0, acc=0, s1=0, s2=0, s2rej=0, err2=0.0, launches=0)
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            st = s.simulate(nsweeps=1, seed=run_seed, check_every=0, delayed=delayed, variant=variant)
            dev += st.seconds
            tot["moves"] += st.moves
            tot["acc"] += st.acc_trans + st.acc_rot
            tot["s1"] += st.da_stage1_rejected
            tot["s2"] += st.da_stage2_tried
            tot["s2rej"] += st.da_stage2_rejected
            tot["err2"] += st.da_err_rms ** 2 * st.da_stage2_tried
            tot["launches"] += st.launches
        tot["rate"] = tot["moves"] / dev
        return tot

    plain = timed(0)
    da = timed(1)
    s.set_surrogate(None)
    sur.close()
    s.close()
    return {"workload": "psc_cpsc_65536", "particles": 65536, "sweeps_timed": steps,
            "kernel_variant": {"plain": variants[0], "delayed": variants[1]},
            "plain_moves_per_s": plain["rate"], "delayed_moves_per_s": da["rate"],
            "speedup": da["rate"] / plain["rate"],
            "acceptance_plain": plain["acc"] / plain["moves"], "acceptance_delayed": da["acc"] / da["moves"],
            "stage1_decided": da["s1"] / da["moves"],
            "stage2_acceptance": 1.0 - da["s2rej"] / max(1, da["s2"]),
            "move_dE_error_rms": math.sqrt(da["err2"] / max(1, da["s2"])),
            "pair_error_vs_fp64": {"rmse": ev["rmse"], "mae": ev["mae"], "max_abs": ev["max_abs"],
                                   "pairs": ev["pairs"]},
            "training": {"samples": tr.samples, "epochs": epochs, "steps": tr.steps, "seconds": tr.seconds,
                         "mse_first_batch": tr.loss_first, "mse_last_batch": tr.loss_last,
                         "collect_seconds": collect_s, "melt_seconds": melt_s, "melt_sweeps": melt}}


def bench_bilayer(steps, seed=1, warm=20):
    """Lipid bilayers: 10,000 three-bead lipids (30,000 particles: SPN head + two TPSC tails,
    bonds k=50 r0=1) in two flat bilayers in a 60x60x40 box, NVT T=1, single-particle moves
    plus N*chainprob (0.1) rigid chain moves per sweep; device-timed, L2 flushed between
    one-sweep steps."""
    import torch

    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.bilayers(50, seed=seed))
    p = s.default_run()
    p.check_every = 0
    p.seed = seed
    s.simulate(p, nsweeps=warm)
    variant = tune_variant(s, p)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    dev = 0.0
    moves = chain = acc = chain_acc = launches = 0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = s.simulate(p, nsweeps=1)
        dev += st.seconds
        moves += st.moves
        chain += st.acc_chain + st.rej_chain
        chain_acc += st.acc_chain
        acc += st.acc_trans + st.acc_rot
        launches += st.launches
    exact = s.all_to_all()
    drift = abs(st.energy - exact)
    s.close()
    return {"workload": "bilayer_30000", "particles": 30000, "chains": 10000, "sweeps_timed": steps,
            "kernel_variant": variant,
            "moves_per_s": (moves + chain) / dev, "particle_moves_per_s": moves / dev,
            "chain_moves_per_s": chain / dev, "acceptance": acc / max(1, moves),
            "chain_acceptance": chain_acc / max(1, chain), "ms_per_sweep": 1e3 * dev / steps,
            "running_energy_error": drift, "launches": launches}


def bench_wl(steps, seed=1, warm=20):
    """Wang-Landau (WangLandau, scOOP/mc/wanglandau.h): a CPSC particle above a bilayer of
    800 three-bead lipids (2401 particles) with adaptive weights over its height relative to
    the system centre and its axis z component (options wlm = 1 3, the reference's membrane
    example), against the same system without the bias, both with cells of the full cut-off
    (the reach Wang-Landau runs choose) and the dataflow sweep; single-particle moves only (a
    chain phase on this small box -- few, crowded chain cells -- would dominate both
    timings); device-timed, L2 flushed between one-sweep steps."""
    import torch

    from sc_gb300 import System, workloads

    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    out = {"workload": "protein_bilayer_2401", "particles": 2401, "order_parameters": [1, 3], "sweeps_timed": steps}
    for key, wlm in (("plain", (0, 0)), ("wang_landau", (1, 3))):
        opts, top, cfg, wl = workloads.protein_bilayer(seed=seed, wlm=wlm, chainprob=0.0)
        s = System.from_text(opts, top, cfg)
        if wlm[0]:
            s.wl_load(text=wl)
        p = s.default_run()
        p.check_every = 0
        p.seed = seed
        p.stencil = 1       # the reach Wang-Landau runs choose (widest cells), for both runs
        p.variant = 4
        s.simulate(p, nsweeps=warm)
        dev = 0.0
        moves = launches = 0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            st = s.simulate(p, nsweeps=1)
            dev += st.seconds
            moves += st.moves + st.acc_chain + st.rej_chain
            launches += st.launches
        out[key + "_moves_per_s"] = moves / dev
        out[key + "_ms_per_sweep"] = 1e3 * dev / steps
        if wlm[0]:
            i = s.wl_info()
            out["alpha"] = i.alpha
            out["bins"] = [i.currorder[0], i.currorder[1]]
            out["launches_per_sweep"] = launches / steps
        s.close()
    out["wl_cost"] = out["plain_moves_per_s"] / out["wang_landau_moves_per_s"]
    try:
        opts, top, cfg, wl = workloads.protein_bilayer(seed=seed, wlm=(1, 3), chainprob=0.0)
        rate, m = wl_cpu_baseline((opts, top, cfg), wl, seed)
        out["cpu_port_moves_per_s"] = rate
        out["cpu_port_sample"] = f"{m} moves, one core (oracle/sc_oracle.cpp or_wl_run: the reference's loop with the bias)"
    except Exception as ex:      # the baseline is reported, not required
        out["cpu_port_moves_per_s"] = None
        out["cpu_port_sample"] = f"failed: {ex}"
    # eight walkers updating one table (the reference's multiple walkers over MPI), moved
    # by the same launches
    from sc_gb300 import ReplicaSet

    nw = 8
    opts, top, cfg, wl = workloads.protein_bilayer(seed=seed, wlm=(1, 3), chainprob=0.0)
    ws = []
    for k in range(nw):
        w = System.from_text(opts, top, cfg)
        w.wl_load(text=wl)
        ws.append(w)
    System.wl_share(ws)
    R = ReplicaSet(ws, temperatures=[1.0] * nw)
    R.run(warm, exchange_every=0, seed=seed, stencil=1, variant=4)
    dev = 0.0
    moves = 0
    for k in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        st, _, _, _, _ = R.run(1, exchange_every=0, seed=seed, stencil=1, variant=4)
        dev += st.seconds
        moves += st.moves
    out["walkers"] = nw
    out["walkers_moves_per_s"] = moves / dev
    out["walkers_gain"] = out["walkers_moves_per_s"] / out["wang_landau_moves_per_s"]
    R.close()
    for w in ws:
        w.close()
    return out


def main():
    a = parse()
    rank, world, local = dist_info()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    if a.only in ("replicas", "surrogate", "bilayer", "wl"):
        if rank == 0:
            fn = {"replicas": bench_replicas, "surrogate": bench_surrogate, "bilayer": bench_bilayer,
                  "wl": bench_wl}[a.only]
            print(json.dumps({a.only: fn(200 if a.only == "replicas" else a.steps, seed=a.seed)}), flush=True)
        return
    import numpy as np
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from sc_gb300 import System  # noqa: F401

    s, texts = open_workload(a.workload, a.seed)
    from sc_gb300 import _lib as L

    L.check(s._lib.sc_set_device(s._h, local))
    n = s.n
    p = s.default_run()
    p.seed = a.seed + 7919 * rank
    p.check_every = 0
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    def l2_flush():
        flush.zero_()
        torch.cuda.synchronize()

    # tuner: the cell-list reach (cell size maxcut/s, (s+1)^3 colours) that moves this
    # system fastest, timed on a few sweeps each
    # (on a copy, so that the measured system starts from the same state as the reference arm)
    # each candidate on a fresh copy of the start (an NPT system compresses while it runs,
    # so one copy moved through all candidates would favour the first ones)
    best = None
    for reach, variant in ((1, 0), (2, 0), (3, 0), (2, 1), (1, 2), (2, 2), (1, 4), (2, 4), (3, 4), (2, 5)):
        tune, _ = open_workload(a.workload, a.seed)
        L.check(tune._lib.sc_set_device(tune._h, local))
        try:
            tune.simulate(p, nsweeps=4, stencil=reach, variant=variant)            # grid, graph capture
            st = tune.simulate(p, nsweeps=10, stencil=reach, variant=variant)
        except Exception:
            tune.close()
            continue
        tune.close()
        rate = st.moves / max(st.seconds, 1e-12)
        if best is None or rate > best[2]:
            best = (reach, variant, rate)
    p.stencil, p.variant = best[0], best[1]
    # warm-up
    s.simulate(p, nsweeps=max(3, a.warmup))
    # the state the timed sweeps start from: the end-to-end leg starts from it as well (an
    # NPT system compresses while it runs, and denser states take longer per sweep)
    start_state, start_box = s.particles(), s.box
    # the timed sweeps also time their move launches with CUDA events on the library's
    # stream (recorded around the launches, read after each sweep: no synchronisation inside)
    p.time_phases = 1
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_s = 0.0
    moves = 0
    launches = 0
    tested = evaluated = 0
    acc = 0
    phase_s, phase_n = 0.0, 0
    for k in range(a.steps):
        l2_flush()
        st = s.simulate(p, nsweeps=1)
        dev_s += st.seconds
        moves += st.moves
        launches += st.launches
        tested += st.pairs_tested
        evaluated += st.pairs_evaluated
        acc += st.acc_trans + st.acc_rot
        phase_s += st.phase_seconds
        phase_n += st.phase_launches
    p.time_phases = 0
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    t_max = max_over_ranks(dev_s, dist, f"cuda:{local}")
    value = moves * world / t_max

    # end to end through the public API with host buffers, from the same start
    state = start_state
    s.box = start_box
    bytes_per_particle = C.sizeof(L.Particle)
    e2e_moves = 0
    t0 = time.perf_counter()
    for k in range(0 if a.no_e2e else a.steps):
        s.set_particles(0, state)                 # host -> device (uploaded by the next call)
        st = s.simulate(p, nsweeps=1)
        state = s.particles()                     # device -> host
        e2e_moves += st.moves
    e2e_s = max(time.perf_counter() - t0, 1e-12)
    e2e = {"value": e2e_moves * world / e2e_s if e2e_moves else None, "unit": UNIT, "h2d_bytes_per_step": n * bytes_per_particle,
           "d2h_bytes_per_step": 2 * n * bytes_per_particle + 64,
           "note": "state passed in and out as host sc_particle arrays around every sweep (staged by the library through pinned host memory)"}

    peaks, peak_kind = measured_peaks()
    # algorithmic bytes of the move kernel: 28 B (position + type) per candidate pair tested
    # (old and new configuration), 24 B axis + 96 B patch vectors per pair evaluated
    bytes_per_launch = (tested * 28 + evaluated * 120) / max(1, phase_n)
    t_launch = phase_s / max(1, phase_n)
    achieved = bytes_per_launch / t_launch / 1e9 if t_launch > 0 else None
    kernel = ["kColour", "kColourDense", None, None, "kColourFlow", "kColourFlowDense"][int(p.variant) & 5]
    roof = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": profiled_traffic(kernel, a.workload),
            "traffic_source": f"profiles/{kernel}_{a.workload}.md (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "avg_launch_us": t_launch * 1e6, "algorithmic_bytes_per_launch": bytes_per_launch,
            "note": "the move kernel is FP64-latency bound; see fp64 for its arithmetic rate"}
    flops_per_launch = (tested * 17 + evaluated * 600) / max(1, phase_n)
    fp64 = {"achieved_tflops": flops_per_launch / t_launch / 1e12 if t_launch > 0 else None,
            "peak_tflops_nominal": 1.25,
            "note": "17 FP64 ops per candidate pair (image + r^2), ~600 per evaluated pair (estimate from the kernel "
                    "source); nominal GB300 FP64 peak, not measured"}

    # CPU baseline: the oracle restatement of the reference loop, one core, bounded sample
    cpu = None
    if rank == 0 and not a.no_cpu:
        try:
            probe_moves, probe_s = cpu_run(texts, a.seed, 1, 400)
            per_move = probe_s / max(1, probe_moves)
            target = int(max(1000, min(50 * n, a.cpu_seconds / per_move)))
            m, sec = cpu_run(texts, a.seed, 100, target)
            cpu = {"value": m / sec, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"{m} moves of {a.workload} from the same start (oracle/sc_oracle.cpp or_mc_run: "
                             f"sequential Metropolis, Verlet list every 10 sweeps, O(N^2) volume move)"}
        except Exception as ex:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {ex}"}

    replicas = surrogate = bilayer = wang_landau = None
    if rank == 0 and a.only == "all" and not a.no_e2e:
        try:
            replicas = bench_replicas(200, seed=a.seed)
        except Exception as ex:
            replicas = {"error": str(ex)}
        try:
            surrogate = bench_surrogate(max(5, a.steps // 2), seed=a.seed)
        except Exception as ex:
            surrogate = {"error": str(ex)}
        try:
            bilayer = bench_bilayer(max(5, a.steps // 2), seed=a.seed)
        except Exception as ex:
            bilayer = {"error": str(ex)}
        try:
            wang_landau = bench_wl(max(5, a.steps // 2), seed=a.seed)
        except Exception as ex:
            wang_landau = {"error": str(ex)}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": 1e3 * t_max / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": a.workload, "n_particles": n, "step": "one sweep (N moves) + volume move",
                           "stencil": int(p.stencil), "kernel_variant": int(p.variant),
                           "parallelism": "replicas" if world > 1 else "single", "l2": "flushed between steps",
                           "seed": a.seed, "plain_fp64": True},
                "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roof, "fp64": fp64,
                "cpu_baseline": cpu, "replicas": replicas, "surrogate": surrogate, "bilayer": bilayer,
                "wang_landau": wang_landau,
                "detail": {"acceptance": acc / max(1, moves), "pairs_tested_per_move": tested / max(1, moves),
                           "pairs_evaluated_per_move": evaluated / max(1, moves)}}
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
