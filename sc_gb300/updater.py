"""The output side of Updater::simulate (scOOP/mc/updater.cpp:45-389) around the GPU move loop.

The reference appends, every `report` sweeps, the exact total energy and the alignment
order to energy.dat and the box volume to stat.dat (updater.cpp:313-318), every `movie`
sweeps a frame to the movie file (Updater::dumpMovie, updater.h:82-93, with Conf::draw,
Conf.h:388-424), and at the end writes config.last (Conf.h:413-422).  With Wang-Landau
weights it also writes the weights file every `report` sweeps (WangLandau::write,
updater.cpp:320-322), stops where the flatness schedule ends the run (updater.cpp:255-265)
and writes the final file (WangLandau::endWangLandau, updater.cpp:388).  With
grand-canonical species it writes top.last with the final counts (main.cpp:313-331).
`run` does the same around blocks of GPU sweeps, in the reference's formats; the blocks
pass their offset in the loop, so that grand-canonical moves fall on the reference's sweeps.
"""
import os

from ._lib import ScError


def _has_wl(system):
    try:
        system.wl_info()
        return True
    except ScError:
        return False


def _frame(system, sweep):
    parts = system.particles()
    box = system.box
    lines = [f"{len(parts)}", f"sweep {sweep}; box {box[0]:.10f} {box[1]:.10f} {box[2]:.10f}"]
    for p in parts:
        # Conf::draw: wrapped real-space position, axis, first patch direction, switched, molType
        x = [box[k] * (p.pos[k] - round(p.pos[k])) for k in range(3)]
        v = list(x) + list(p.dir) + list(p.patchdir[0])
        lines.append("%15.8e %15.8e %15.8e   %15.8e %15.8e %15.8e   %15.8e %15.8e %15.8e %d %d" % (*v, 0, p.molType))
    return "\n".join(lines) + "\n"


def run(system, nsweeps, report=0, movie=0, directory=".", params=None, wl_file="wl-new.dat", nequil=0, adjust=0,
        **overrides):
    """Runs nsweeps sweeps on the GPU, writing energy.dat / stat.dat every `report` sweeps,
    movie frames every `movie` sweeps and config.last at the end (and, with Wang-Landau
    weights, `wl_file`).  With nequil > 0 an equilibration comes first, as in main.cpp:270-287:
    nequil/2 sweeps with the maximum steps adjusted every `adjust` sweeps, nequil/2 without,
    then config.eq (Conf::draw with the box line).  Returns the summed stats counters (moves,
    acceptances) of the production blocks and the sweeps run."""
    p = params if params is not None else system.default_run()
    for k, v in overrides.items():
        setattr(p, k, v)
    eq_sweeps = 0
    if nequil > 0:
        est = system.equilibrate(nequil, adjust, params=p)
        eq_sweeps = est.sweeps
        system.write_config(os.path.join(directory, "config.eq"))
        p.edge_mx = system.default_run().edge_mx       # the adapted box edge range
    ef = os.path.join(directory, "energy.dat")
    sf = os.path.join(directory, "stat.dat")
    mf = os.path.join(directory, "movie")
    # Updater::emptyFiles writes the headers (updater.cpp:77-85)
    with open(ef, "w") as f:
        f.write("# sweep    energy\n")
    with open(sf, "w") as f:
        f.write("# sweep    volume\n")
    if movie:
        open(mf, "w").close()
    wl = _has_wl(system)
    wf = os.path.join(directory, wl_file)
    totals = {}
    sweep = 0
    next_dump = report if report > 0 else None
    next_frame = movie if movie > 0 else None
    while sweep < nsweeps:
        stops = [nsweeps] + [x for x in (next_dump, next_frame) if x]
        block = min(stops) - sweep
        st = system.simulate(p, nsweeps=block, sweep_offset=sweep)
        for name, _ in type(st)._fields_:
            if name.startswith(("acc_", "rej_", "moves", "pairs_")):
                totals[name] = totals.get(name, 0) + getattr(st, name)
        sweep += st.sweeps
        if st.sweeps < block:           # Wang-Landau converged: the reference stops here
            break
        if next_dump and sweep == next_dump:
            box = system.box
            with open(sf, "a") as f:
                f.write(" %d; %.10f\n" % (sweep, box[0] * box[1] * box[2]))
            with open(ef, "a") as f:
                f.write(" %d; %.10f  %f \n" % (sweep, system.all_to_all(), system.alignment_order()))
            if wl:
                system.wl_write(wf)
            next_dump += report
        if next_frame and sweep == next_frame:
            with open(mf, "a") as f:
                f.write(_frame(system, sweep))
            next_frame += movie
    system.write_config(os.path.join(directory, "config.last"))
    grand = system.grand_stats()
    if grand:
        system.write_top_last(os.path.join(directory, "top.last"))
        # Updater::simulate's closing report of each species (updater.cpp:358-373)
        totals["grand"] = [dict(mol_type=g.mol_type, count=g.count, steps=g.steps, ins_acc=g.ins_acc,
                                ins_rej=g.ins_rej, del_acc=g.del_acc, del_rej=g.del_rej,
                                average_particles=g.average_particles) for g in grand]
    if wl:
        system.wl_end(wf)
    totals["sweeps"] = sweep
    totals["equilibration_sweeps"] = eq_sweeps
    return totals
