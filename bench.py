#!/usr/bin/env python3
"""Benchmark: attempted Metropolis moves per second on one GB300.

Workload (default): psc_cpsc_65536 -- 65,536 patchy spherocylinders, half PSC (patch 90
deg) and half CPSC (cylindrical patch 120 deg), length 3, eps 1, packing fraction 0.2,
NVT T = 1, from a seeded aligned lattice start (sc_gb300/workloads.py).  A step is one
sweep: N attempted single-particle moves (displacements and rotations) on the
checkerboard, all through the C ABI, with the launch shape the library's tuner (sc_tune)
picks on the start.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-timed moves/s of the plain FP64 kernel (CUDA
events on the library's stream, L2 flushed between steps); `e2e` is the same metric
through the public API with host buffers (state uploaded before and downloaded after
every step); `delayed_acceptance` gives the surrogate two-stage moves on the same system
after a melt.  `--impl reference` times the reference's own algorithm (the sequential
loop with its Verlet list, restated in oracle/sc_oracle.cpp and built -Ofast, calibrated
against the reference's own -Ofast binary by tests/test_cpu_baseline.py) on all host cores,
independent seeds per core, on the same workload, set-up outside the timed region.

Sections of the same line (rank 0, default run): `surrogate` (plain against delayed
acceptance with the network trained in the run, after a melt), `mixture` (the
4000-particle NPT binary mixture with one host core of the reference's loop beside it),
`replicas` (64 uneven parallel-tempering replicas in one batch against the same replicas
one after another, and one host core of the reference's loop over the ladders' systems),
`bilayer` (30,000-particle lipid bilayers with chain moves, and one host core of the
reference's loop on them), `wang_landau` (a particle above a bilayer with and without Wang-Landau weights, eight
walkers sharing one table, and the reference's loop with the bias as the CPU baseline).
`--only <section>` runs one of them alone.
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
WORKLOAD = "psc_cpsc_65536"


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
    ap.add_argument("--only", default="all", choices=["all", "main", "replicas", "surrogate", "bilayer", "wl", "mixture"],
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


def wl_cpu_baseline(texts, wl_text, seed, max_moves=3000):
    """One core of the oracle's sequential loop with the Wang-Landau bias (or_wl_run, the
    reference's partDisplace / partRotate with WangLandau::run / runRot) on a bounded
    sample of the same system and weights: moves/s."""
    import numpy as np

    import oracle_ffi as O

    opts, top, cfg = texts
    ts = O.TextSystem(opts, top, cfg)
    sysm, o = ts.sys, ts.opts
    o.seed = seed
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
    st.wlmtype = -1
    if O.lib().or_wl_orders(C.byref(sysm), st.wlm, -1, st.minorder, st.dorder, cur, cm, C.byref(sv)) != 0:
        raise RuntimeError("oracle: order parameters outside its restatement")
    st.cur[0], st.cur[1] = cur[0], cur[1]
    o.nsweeps, o.max_moves = 1 << 30, max_moves
    ms = O.McStats()
    O.lib(fast=True).or_wl_run(C.byref(sysm), C.byref(o), C.byref(st), C.byref(ms))
    return ms.moves / max(ms.seconds, 1e-12), ms.moves


REF_MAXN = 30003      # MAXN of the reference (scOOP/structures/macros.h:60)


def bilayer_cpu_baseline(texts, seed, seconds=8.0):
    """The reference's loop on one host core for the 30,000-particle bilayers: particle and
    chain moves (chainprob of the options), the -Ofast restatement with TotalEFull and the
    Verlet list every 10 sweeps (the reference's energy matrix would take 3.6 GB and an O(N^2)
    set-up of unfiltered chain pairs), set-up outside the timing, a bounded sample of moves."""
    import oracle_ffi as O

    ts = O.TextSystem(*texts)
    run = O.McRun(ts, seed=seed, energy_matrix=False, fast=True)
    probe = run.advance(2000)
    rate = probe.moves / max(probe.seconds, 1e-9)
    m0, s0, c0 = run.stats.moves, run.stats.seconds, run.stats.acc_chain + run.stats.rej_chain
    st = run.advance(max(2000, int(seconds * rate)))
    moves, secs = st.moves - m0, st.seconds - s0
    chains = st.acc_chain + st.rej_chain - c0
    setup = run.setup_seconds
    run.close()
    return {"value": moves / max(secs, 1e-9), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{moves} moves ({chains} of them chain moves) of bilayer_30000 by the reference's sequential "
                      f"loop restated in oracle/sc_oracle.cpp, built -Ofast (TotalEFull, Verlet list every 10 "
                      f"sweeps); set-up ({setup:.1f} s: initial energy, first pair list) outside the timing"}


def replicas_cpu_baseline(systems, temps, seed, seconds=8.0):
    """The reference's loop on one host core for the parallel-tempering replicas: each
    ladder's system at one of its temperatures (cycling through the ladder), the -Ofast
    restatement with the reference's defaults (TotalEMatrix, Verlet list every 10 sweeps),
    set-up outside the timing, a bounded sample of moves each.  Without MPI the reference runs
    its replicas as independent processes (no exchange); one core moving all of them one
    after another, each for the same number of sweeps, makes sum(N) moves per sum(N / rate)
    seconds, which is the rate returned."""
    import oracle_ffi as O

    budget = seconds / len(systems)
    work = time_ = 0.0
    moves = 0
    for g, texts in enumerate(systems):
        ts = O.TextSystem(*texts)
        ts.opts.temper = float(temps[g % len(temps)])
        n = ts.sys.n
        run = O.McRun(ts, seed=seed + 77 * g, energy_matrix=n <= REF_MAXN, fast=True)
        probe = run.advance(min(n, 1000))
        rate = probe.moves / max(probe.seconds, 1e-9)
        m0, s0 = run.stats.moves, run.stats.seconds
        st = run.advance(max(n, int(budget * rate)))
        rate = (st.moves - m0) / max(st.seconds - s0, 1e-9)
        moves += st.moves - m0
        work += n
        time_ += n / rate
        run.close()
    return {"value": work / time_, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{moves} moves over the {len(systems)} ladders' systems (one temperature each) of the "
                      f"reference's sequential loop restated in oracle/sc_oracle.cpp, built -Ofast (TotalEMatrix, "
                      f"Verlet list every 10 sweeps), set-up outside the timing; the 64 replicas one after another"}


def _ref_worker(texts, seed, energy_matrix, probe_moves, warmup_steps, steps, step_moves, barrier, out):
    """One host core running the reference's loop (the oracle's restatement at -Ofast) on its
    own copy of the start: set-up, probe, warm-up and timed phases separated by barriers, so
    that the caller's clock covers the timed moves only."""
    import oracle_ffi as O

    ts = O.TextSystem(*texts)
    run = O.McRun(ts, seed=seed, energy_matrix=energy_matrix, fast=True)
    st = run.advance(probe_moves)
    out.put(("probe", st.moves / max(st.seconds, 1e-9), run.setup_seconds))
    barrier.wait()                       # the caller sizes the steps from the probes
    sm = step_moves.value
    run.advance(sm * warmup_steps)
    barrier.wait()                       # timed region starts
    m0 = run.stats.moves
    run.advance(sm * steps)
    moves = run.stats.moves - m0
    barrier.wait()                       # timed region ends
    st = run.stats
    out.put(("done", moves, (st.acc_trans + st.acc_rot) / max(1, st.moves), st.moves))
    run.close()


def _neighbours_estimate(texts):
    """Particles within the reference's pair-list cutoff of one particle (main.cpp:117-126)."""
    import oracle_ffi as O

    opts, top, cfg = texts
    o = O.parse_options(opts)
    box = [float(x) for x in cfg.strip().splitlines()[0].split()[:3]]
    n = cfg.count("\n") - 1
    rc = 2.0 * float(o.get("transmx", "0")) * (1 + int(o.get("pairlist_update", "0"))) * 2 + 5.0
    return min(n, n / (box[0] * box[1] * box[2]) * 4.0 / 3.0 * math.pi * rc ** 3)


def cpu_reference_rate(texts, cores, warmup_steps, steps, seed, seconds_budget):
    """Moves/s of the reference's own algorithm on `cores` host cores: independent seeds, one
    process each, timed between barriers after every process has set up its system (initial
    energy / energy matrix, first pair list: what precedes the reference's timed loop).  The
    energy calculator is the reference's default TotalEMatrix when N fits its MAXN, else
    TotalEFull, both with the Verlet list every pairlist_update sweeps.  A step is at most one
    sweep per process, sized so that warm-up plus timed steps take about seconds_budget; the
    process count is bounded by the host memory the pair lists need."""
    import multiprocessing as mp

    n = texts[2].count("\n") - 1
    matrix = n <= REF_MAXN
    per = 8.0 * n * _neighbours_estimate(texts) + (8.0 * n * n if matrix else 0.0) + 64e6
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
        cores = max(1, min(cores, int(0.5 * avail / per)))
    except (ValueError, OSError):
        pass
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(cores + 1)
    out = ctx.Queue()
    step_moves = ctx.Value("l", n)
    probe = min(n, 2000)
    procs = [ctx.Process(target=_ref_worker, args=(texts, seed + 1000 + k, matrix, probe, warmup_steps, steps,
                                                   step_moves, barrier, out)) for k in range(cores)]
    for q in procs:
        q.start()
    limit = 1800.0                       # a process that died must not hang the caller
    try:
        rates, setups = [], []
        for _ in range(cores):
            tag, rate, setup = out.get(timeout=limit)
            rates.append(rate)
            setups.append(setup)
        per_step = seconds_budget / max(1, warmup_steps + steps)
        step_moves.value = int(max(200, min(n, per_step * min(rates))))
        barrier.wait(timeout=limit)      # probes done, step size set
        barrier.wait(timeout=limit)      # warm-up done
        t0 = time.perf_counter()
        barrier.wait(timeout=limit)      # timed moves done
        wall = time.perf_counter() - t0
        moves = 0
        acc = []
        for _ in range(cores):
            tag, m, a, _tot = out.get(timeout=limit)
            moves += m
            acc.append(a)
    finally:
        for q in procs:
            q.join(timeout=5)
            if q.is_alive():
                q.kill()
    return {"value": moves / wall, "moves": moves, "seconds": wall, "cores": cores, "step_moves": step_moves.value,
            "energy_calculator": "TotalEMatrix" if matrix else "TotalEFull", "setup_seconds": max(setups),
            "acceptance": float(sum(acc) / len(acc))}


def _reference_sample(r, workload, steps):
    return (f"{r['cores']} processes x {steps} steps x {r['step_moves']} moves of {workload} (independent seeds; "
            f"the reference's sequential loop restated in oracle/sc_oracle.cpp, built -Ofast: Verlet list every 10 "
            f"sweeps, {r['energy_calculator']}, O(N^2) volume move with probability shave/N per move); set-up "
            f"({r['setup_seconds']:.1f} s: initial energy, first pair list) outside the timed region; calibrated "
            f"within 15 % of the reference's own -Ofast binary (tests/test_cpu_baseline.py)")


def run_reference(a, rank, world):
    """CPU arm: the reference's loop on all host cores, same workload, metric and unit."""
    if rank != 0:
        return
    from sc_gb300 import workloads

    texts = workloads.WORKLOADS[a.workload](a.seed)
    n = texts[2].count("\n") - 1
    cores = os.cpu_count() or 1
    r = cpu_reference_rate(texts, cores, a.warmup, a.steps, a.seed, seconds_budget=120.0)
    value = r["value"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * r["seconds"] / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": a.workload, "n_particles": n, "seed": a.seed, "cores": r["cores"],
                       "step": f"{r['step_moves']} moves per process"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": r["cores"], "kind": "port",
                             "sample": _reference_sample(r, a.workload, a.steps)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": {"acceptance": r["acceptance"], "timed_seconds": r["seconds"], "moves": r["moves"]}}
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
    solo = s1.tune(s1.default_run(), sweeps=3)[0].variant
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
    try:
        cpu = replicas_cpu_baseline(systems, temps, seed)
    except Exception as ex:                 # the oracle is not built: the section stands without it
        cpu = {"error": str(ex)}
    return {"workload": "pt64_psc_uneven", "replicas": len(ctxs), "particles": particles, "stencil": best[0],
            "kernel_variant": {"batched": best[1], "plain": solo},
            "batched_moves_per_s": batched, "plain_moves_per_s": plain, "speedup": batched / plain,
            "cpu_baseline": cpu, "speedup_vs_cpu_core": batched / cpu["value"] if "value" in cpu else None,
            "batched_delayed_moves_per_s": batched_da, "speedup_batched_delayed": batched_da / plain,
            "delayed_stage1_decided": std.da_stage1_rejected / max(1, std.moves),
            "exchanges_tried": int(tried.sum()), "exchange_acceptance": float(acc.sum() / max(1, tried.sum())),
            "sweeps": steps}


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
    # each mode its fastest launch shape (the library's tuner; later runs pass variant = -1)
    variants = {d: s.tune(pt, sweeps=4, delayed=d)[0] for d in (0, 1)}

    def timed(delayed):
        variant = -1
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
            "kernel_variant": {"plain": variants[0].variant, "delayed": variants[1].variant},
            "stencil": {"plain": variants[0].stencil, "delayed": variants[1].stencil},
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
    best, _ = s.tune(p, sweeps=4)
    variant = best.variant
    p.variant = -1
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
    try:
        cpu = bilayer_cpu_baseline(workloads.bilayers(50, seed=seed), seed)
    except Exception as ex:                 # the oracle is not built: the section stands without it
        cpu = {"error": str(ex)}
    return {"workload": "bilayer_30000", "particles": 30000, "chains": 10000, "sweeps_timed": steps,
            "kernel_variant": variant, "cpu_baseline": cpu,
            "speedup_vs_cpu_core": (moves + chain) / dev / cpu["value"] if "value" in cpu else None,
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


def fp64_peak(device):
    """This GPU's FP64 rates from the library's probe kernels (sc_fp64_rates)."""
    from sc_gb300 import _lib as L

    lib = L.load()
    v = [C.c_double() for _ in range(4)]
    L.check(lib.sc_fp64_rates(device, *[C.byref(x) for x in v]))
    return {"dmul_dadd_ops_per_s": v[0].value, "one_lane_ops_per_s": v[1].value, "dfma_flops": v[2].value,
            "latency_cycles": v[3].value}


def timed_sweeps(s, p, steps, flush, dist=None, clocks=None):
    """`steps` one-sweep steps, device-timed (CUDA events on the library's stream), L2 flushed
    before each; the move launches are timed too (events recorded around them, read after the
    sweep).  Returns the totals."""
    import torch

    p.time_phases = 1
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    tot = dict(seconds=0.0, moves=0, launches=0, tested=0, evaluated=0, acc=0, phase_s=0.0, phase_n=0)
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = s.simulate(p, nsweeps=1)
        tot["seconds"] += st.seconds
        tot["moves"] += st.moves
        tot["launches"] += st.launches
        tot["tested"] += st.pairs_tested
        tot["evaluated"] += st.pairs_evaluated
        tot["acc"] += st.acc_trans + st.acc_rot
        tot["phase_s"] += st.phase_seconds
        tot["phase_n"] += st.phase_launches
    p.time_phases = 0
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    tot["clocks"] = clocks.stop() if clocks else None
    return tot


KERNELS = {0: "kColour", 1: "kColourDense", 2: "kColour", 3: "kColourDense", 4: "kColourFlow", 5: "kColourFlowDense",
           6: "kColourFlow", 7: "kColourFlowDense"}


def roofline(tot, variant, workload, peaks, peak_kind, fp64):
    """The move kernel against the HBM roofline (algorithmic bytes: 28 B position + type per
    candidate pair tested, old and new configuration, 120 B axis + patch vectors per pair
    evaluated) and against this GPU's measured FP64 instruction rate (17 FP64 operations per
    candidate pair for the image and r^2, ~600 per evaluated pair, counted from the kernel
    source)."""
    n = max(1, tot["phase_n"])
    t_launch = tot["phase_s"] / n
    bytes_per_launch = (tot["tested"] * 28 + tot["evaluated"] * 120) / n
    achieved = bytes_per_launch / t_launch / 1e9 if t_launch > 0 else None
    kernel = ("kCellWarpsFlowDense" if variant & 1 else "kCellWarpsFlow") if variant & 8 else KERNELS[int(variant) & 7]
    roof = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": profiled_traffic(kernel, workload),
            "traffic_source": f"profiles/{kernel}_{workload}.md (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "avg_launch_us": t_launch * 1e6, "algorithmic_bytes_per_launch": bytes_per_launch,
            "note": "the move kernel is bound by FP64 latency, not by HBM: see fp64"}
    ops = (tot["tested"] * 17 + tot["evaluated"] * 600) / n
    fp = {"achieved_ops_per_s": ops / t_launch if t_launch > 0 else None,
          "note": "17 FP64 operations per candidate pair (image + r^2), ~600 per evaluated pair (counted from the "
                  "kernel source); peaks from the library's own probe kernels on this GPU (sc_fp64_rates)"}
    if fp64:
        fp.update({"peak_ops_per_s": fp64["dmul_dadd_ops_per_s"], "frac": fp["achieved_ops_per_s"] /
                   fp64["dmul_dadd_ops_per_s"] if fp["achieved_ops_per_s"] else None,
                   "peak_dfma_tflops": fp64["dfma_flops"] / 1e12, "one_lane_ops_per_s": fp64["one_lane_ops_per_s"],
                   "dependent_latency_cycles": fp64["latency_cycles"]})
    return roof, fp


def bench_mixture(steps, seed=1, cpu_seconds=15.0):
    """The 4000-particle NPT binary mixture (2000 CPSC + 2000 SPA, P* = 0.5, one isotropic
    volume move per sweep): device-timed plain sweeps (library tuner) and one host core of
    the reference's loop (the reference's energy matrix) from the same start."""
    import torch

    from sc_gb300 import System, workloads

    texts = workloads.npt_cpsc_spa(4000, seed=seed)
    s = System.from_text(*texts)
    p = s.default_run()
    p.seed, p.check_every = seed, 0
    best, rates = s.tune(p, sweeps=8)
    p.variant = -1
    s.simulate(p, nsweeps=5)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    tot = timed_sweeps(s, p, steps, flush)
    s.close()
    out = {"workload": "npt_cpsc_spa_4000", "particles": 4000, "sweeps_timed": steps,
           "stencil": best.stencil, "kernel_variant": best.variant,
           "moves_per_s": tot["moves"] / tot["seconds"], "ms_per_sweep": 1e3 * tot["seconds"] / steps,
           "pair_evaluations_per_s": tot["evaluated"] / tot["seconds"]}
    try:
        r = cpu_reference_rate(texts, 1, 1, 3, seed, seconds_budget=cpu_seconds)
        out["cpu_baseline"] = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": _reference_sample(r, "npt_cpsc_spa_4000", 3)}
    except Exception as ex:
        out["cpu_baseline"] = {"value": None, "sample": f"failed: {ex}"}
    return out


def main():
    a = parse()
    rank, world, local = dist_info()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    if a.only in ("replicas", "surrogate", "bilayer", "wl", "mixture"):
        if rank == 0:
            fn = {"replicas": bench_replicas, "surrogate": bench_surrogate, "bilayer": bench_bilayer,
                  "wl": bench_wl, "mixture": bench_mixture}[a.only]
            print(json.dumps({a.only: fn(200 if a.only == "replicas" else a.steps, seed=a.seed)}), flush=True)
        return
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from sc_gb300 import _lib as L

    s, texts = open_workload(a.workload, a.seed)
    L.check(s._lib.sc_set_device(s._h, local))
    n = s.n
    p = s.default_run()
    p.seed = a.seed + 7919 * rank
    p.check_every = 0
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

    # the library's tuner (sc_tune): every cell reach and kernel variant timed on the start,
    # which it restores; the runs below use its choice (variant = -1)
    best, rates = s.tune(p, sweeps=6)
    p.variant = -1
    s.simulate(p, nsweeps=max(3, a.warmup))          # warm-up
    # the state the timed sweeps start from: the end-to-end leg starts from it as well
    start_state, start_box = s.particles(), s.box
    tot = timed_sweeps(s, p, a.steps, flush, dist, Clocks(local))
    t_max = max_over_ranks(tot["seconds"], dist, f"cuda:{local}")
    value = tot["moves"] * world / t_max

    # end to end through the public API with host buffers, from the same start
    state = start_state
    s.box = start_box
    bytes_per_particle = C.sizeof(L.Particle)
    e2e_moves = 0
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for k in range(0 if a.no_e2e else a.steps):
        s.set_particles(0, state)                 # host -> device (uploaded by the next call)
        st = s.simulate(p, nsweeps=1)
        state = s.particles(out=state)            # device -> host, into the caller's buffer
        e2e_moves += st.moves
    e2e_s = max_over_ranks(max(time.perf_counter() - t0, 1e-12), dist, f"cuda:{local}")
    e2e = {"value": e2e_moves * world / e2e_s if e2e_moves else None, "unit": UNIT,
           "h2d_bytes_per_step": n * bytes_per_particle, "d2h_bytes_per_step": 2 * n * bytes_per_particle + 64,
           "note": "state passed in and out as host sc_particle arrays around every sweep (staged by the library "
                   "through pinned host memory); the library recomputes the exact energy after each host change"}

    peaks, peak_kind = measured_peaks()
    fp64_err = None
    try:
        fp64 = fp64_peak(local)
    except Exception as ex:
        fp64, fp64_err = None, str(ex)
    roof, fp = roofline(tot, best.variant, a.workload, peaks, peak_kind, fp64)
    if fp64_err:
        fp["error"] = fp64_err

    # CPU baseline: one host core of the reference's loop on a bounded sample of the same start
    cpu = None
    if rank == 0 and not a.no_cpu:
        try:
            r = cpu_reference_rate(texts, 1, 1, 3, a.seed, seconds_budget=a.cpu_seconds)
            cpu = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": _reference_sample(r, a.workload, 3)}
        except Exception as ex:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {ex}"}

    sections = {}
    if rank == 0 and a.only == "all" and not a.no_e2e:
        for key, fn, steps in (("surrogate", bench_surrogate, max(5, a.steps // 2)),
                               ("mixture", bench_mixture, max(10, a.steps)),
                               ("replicas", bench_replicas, 200),
                               ("bilayer", bench_bilayer, max(5, a.steps // 2)),
                               ("wang_landau", bench_wl, max(5, a.steps // 2))):
            try:
                sections[key] = fn(steps, seed=a.seed)
            except Exception as ex:
                sections[key] = {"error": str(ex)}
    if rank == 0:
        sur = sections.get("surrogate") or {}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": 1e3 * t_max / a.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": a.workload, "n_particles": n, "step": "one sweep (N attempted moves)",
                           "start": "aligned lattice start after the warm-up sweeps",
                           "stencil": int(best.stencil), "kernel_variant": int(best.variant),
                           "parallelism": "replicas" if world > 1 else "single", "l2": "flushed between steps",
                           "seed": a.seed, "plain_fp64": True},
                "clocks": tot["clocks"], "e2e": e2e, "gpu_launches": tot["launches"], "roofline": roof, "fp64": fp,
                "cpu_baseline": cpu,
                "pairs": {"evaluated_per_s": tot["evaluated"] / tot["seconds"],
                          "tested_per_s": tot["tested"] / tot["seconds"],
                          "evaluated_per_move": tot["evaluated"] / max(1, tot["moves"]),
                          "tested_per_move": tot["tested"] / max(1, tot["moves"])},
                "delayed_acceptance": {k: sur.get(k) for k in ("plain_moves_per_s", "delayed_moves_per_s", "speedup",
                                                               "stage1_decided", "workload")} if sur else None,
                "tuner": {"candidates_moves_per_s": rates},
                "detail": {"acceptance": tot["acc"] / max(1, tot["moves"])}}
        line.update(sections)
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
