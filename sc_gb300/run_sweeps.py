"""Run device sweeps of a seeded benchmark system with a chosen launch shape.

    python -m sc_gb300.run_sweeps --workload psc_cpsc --n 16384 --variant 8 --stencil 1 \\
        --warmup 2 --sweeps 1

Prints one JSON line (moves/s of the timed sweeps, device time, launches).  The launch
shape is fixed by the arguments (no tuner), so that a profiler can select the move kernel's
launches by name and position: with --warmup W the timed sweeps' move launches come after
W launches of the same kernel.

    python -m sc_gb300.run_sweeps --workload psc_cpsc --n 65536 --variant 8 --stencil 3 \
        --energy-calls 3

instead makes K calls of sc_simulate with no sweeps, setting the particles again before
each, so that every call recomputes the exact total energy over the cell list (one
kCellEnergy launch per call, as the end-to-end leg of the bench does every step), and
prints the device seconds of each call.
"""
import argparse
import json

from . import System, workloads

BUILDERS = {
    "psc_cpsc": lambda n, seed: workloads.psc_cpsc(n, phi=0.2, seed=seed),
    "npt_cpsc_spa": lambda n, seed: workloads.npt_cpsc_spa(n, seed=seed),
    "nvt_psc": lambda n, seed: workloads.nvt_psc(n, seed=seed),
    "bilayers": lambda n, seed: workloads.bilayers(max(1, int(round((n / 12) ** 0.5))), seed=seed),
    "psc_grand_switch": lambda n, seed: workloads.nvt_psc_grand_switch(n, seed=seed),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="psc_cpsc", choices=sorted(BUILDERS))
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--variant", type=int, default=4)
    ap.add_argument("--stencil", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--sweeps", type=int, default=1)
    ap.add_argument("--energy-calls", type=int, default=0,
                    help="K calls without sweeps, each recomputing the exact energy after a host change")
    a = ap.parse_args()
    s = System.from_text(*BUILDERS[a.workload](a.n, a.seed))
    p = s.default_run()
    p.check_every = 0
    p.variant, p.stencil, p.seed = a.variant, a.stencil, a.seed
    if a.energy_calls > 0:
        parts = s.particles()
        seconds = []
        for _ in range(a.energy_calls):
            s.set_particles(0, parts)           # the host copy is newer: the next call uploads it
            st = s.simulate(p, nsweeps=0)       # and recomputes the exact energy
            seconds.append(st.seconds)
        print(json.dumps({"workload": a.workload, "n": s.n, "variant": a.variant, "stencil": a.stencil,
                          "energy_calls": a.energy_calls, "seconds": seconds, "energy": st.energy}))
        s.close()
        return
    for _ in range(a.warmup):
        s.simulate(p, nsweeps=1)
    st = s.simulate(p, nsweeps=a.sweeps)
    print(json.dumps({"workload": a.workload, "n": s.n, "variant": a.variant, "stencil": a.stencil,
                      "sweeps": a.sweeps, "moves_per_s": st.moves / max(st.seconds, 1e-12), "seconds": st.seconds,
                      "launches": st.launches, "phase_launches": st.phase_launches}))
    s.close()


if __name__ == "__main__":
    main()
