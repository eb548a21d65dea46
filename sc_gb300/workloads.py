"""Seeded synthetic systems in the reference's input format (options, top.init, config.init).

The benchmark systems are described by their physics only (no dataset is
involved); these generators build them deterministically from a seed:
random, non-overlapping centres (closest segment distance >= sigma) and uniform
random orientations, patch vectors perpendicular to the axis.

  npt_cpsc_spa_4000   2000 CPSC (L=3, patch 120 deg) + 2000 SPA (sigma 1, eps 0.5, range 1.5),
                      P*=0.5, T=1, isotropic volume move every sweep
  nvt_psc_1000        1000 PSC (L=3, patch 90 deg, switch 10 deg, eps 1, range 1.12 + 0.2),
                      packing fraction 0.1, T=1
  psc_cpsc_65536      65,536 PSC/CPSC 50/50 at packing fraction 0.2, T=1
"""
import math

import numpy as np

OPTION_DEFAULTS = dict(
    ptype=1, press=0.0, paralpress=0.0, shave=0, nequil=0, adjust=0, nsweeps=100, paramfrq=0, report=0,
    nrepchange=0, nGrandCanon=0, nClustMove=0, movie=0, chainprob=0.0, transmx=0.3, rotmx=20.0,
    edge_mx=0.0, chainmmx=0.0, chainrmx=0.0, temper=1.0, paraltemper=1.0, wlm=0, wlmtype=0,
    switchprob=0.0, pairlist_update=10, seed=1, write_cluster=0)


def options_text(**kw):
    d = dict(OPTION_DEFAULTS)
    d.update(kw)
    d["paraltemper"] = d["temper"]
    return "".join(f"{k} = {v}\n" for k, v in d.items())


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _perp(rng, d):
    v = _unit(rng, len(d))
    v -= (v * d).sum(1, keepdims=True) * d
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _segdist(p1, d1, h1, P2, D2, H2):
    """Closest distance between segment (p1, d1, half-length h1) and segments (P2, D2, H2), vectorised."""
    r = p1[None, :] - P2
    a = np.full(len(P2), 1.0)
    b = (D2 @ d1)
    c = np.full(len(P2), 1.0)
    dd = r @ d1
    e = (r * D2).sum(1)
    den = a * c - b * b
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.where(den > 1e-12, (b * e - c * dd) / den, 0.0)
    s = np.clip(s, -h1, h1)
    t = np.clip(b * s + e, -H2, H2)
    s = np.clip(b * t - dd, -h1, h1)
    t = np.clip(b * s + e, -H2, H2)
    diff = r + s[:, None] * d1[None, :] - t[:, None] * D2
    return np.sqrt((diff * diff).sum(1))


def place(rng, halfl, box, dmin=1.0, max_tries=200000):
    """Random sequential placement; halfl[k] is the half-length of particle k (0 for spheres)."""
    n = len(halfl)
    pos = np.zeros((n, 3))
    dirs = _unit(rng, n)
    cell = max(2.0 * max(halfl) + dmin, dmin) + 1e-9
    nc = np.maximum((box // cell).astype(int), 1)
    grid = {}
    placed = 0
    tries = 0
    while placed < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("placement failed: density too high")
        p = rng.uniform(0, 1, 3) * box
        key = tuple((p / box * nc).astype(int) % nc)
        near = []
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    near += grid.get(((key[0] + dx) % nc[0], (key[1] + dy) % nc[1], (key[2] + dz) % nc[2]), [])
        if near:
            idx = np.array(sorted(set(near)))
            r = pos[idx] - p
            r -= box * np.round(r / box)
            q = p + r
            dist = _segdist(p, dirs[placed], halfl[placed], q, dirs[idx], np.asarray(halfl)[idx])
            if np.any(dist < dmin):
                dirs[placed] = _unit(rng, 1)[0]
                continue
        pos[placed] = p
        grid.setdefault(key, []).append(placed)
        placed += 1
    return pos, dirs, _perp(rng, dirs)


def config_text(box, pos, dirs, pds):
    lines = ["%.17g %.17g %.17g" % tuple(box)]
    for p, d, q in zip(pos, dirs, pds):
        lines.append("%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g 0" % (*p, *d, *q))
    return "\n".join(lines) + "\n"


def _vol_sc(L, sigma=1.0):
    return math.pi / 6 * sigma ** 3 + math.pi / 4 * sigma ** 2 * L


def npt_cpsc_spa(n=4000, phi=0.1, seed=1, press=0.5, temper=1.0):
    L = 3.0
    nc = n // 2
    ns = n - nc
    vol = nc * _vol_sc(L) + ns * math.pi / 6
    box = np.full(3, (vol / phi) ** (1 / 3))
    rng = np.random.default_rng(seed)
    halfl = [L / 2] * nc + [0.0] * ns
    pos, dirs, pds = place(rng, halfl, box)
    top = ("[Types]\n"
           "C 1 CPSC 1.0 1.0 1.12 0.2 120.0 10.0 3.0 0.0\n"
           "A 2 SPA 0.5 1.0 1.1225 0.3775\n"
           "[Molecules]\nC: {\nparticles: 1\n}\nA: {\nparticles: 2\n}\n"
           f"[System]\nC {nc}\nA {ns}\n")
    opts = options_text(ptype=1, press=press, shave=1, edge_mx=0.4, transmx=0.4, rotmx=30.0, temper=temper,
                        seed=seed)
    return opts, top, config_text(box, pos, dirs, pds)


def nvt_psc(n=1000, phi=0.1, seed=1, temper=1.0):
    L = 3.0
    box = np.full(3, (n * _vol_sc(L) / phi) ** (1 / 3))
    rng = np.random.default_rng(seed)
    pos, dirs, pds = place(rng, [L / 2] * n, box)
    top = ("[Types]\nP 1 PSC 1.0 1.0 1.12 0.2 90.0 10.0 3.0 0.0\n"
           f"[Molecules]\nP: {{\nparticles: 1\n}}\n[System]\nP {n}\n")
    opts = options_text(ptype=0, transmx=0.4, rotmx=30.0, temper=temper, seed=seed)
    return opts, top, config_text(box, pos, dirs, pds)


def _lattice(rng, n, phi, L=3.0):
    """Aligned start: axes within 0.1 rad of z on a lattice of layers (random patch
    directions); reaches the densities random sequential placement cannot."""
    edge = (n * _vol_sc(L) / phi) ** (1 / 3)
    nz = max(1, int(edge // (L + 1.05)))
    nxy = int(math.ceil(math.sqrt(n / nz)))
    if edge / nxy < 1.05 + 0.35:
        raise RuntimeError("lattice start: density too high")
    box = np.full(3, edge)
    sites = np.array([(i, j, k) for k in range(nz) for j in range(nxy) for i in range(nxy)], float)
    sites = sites[rng.permutation(len(sites))[:n]]
    pos = (sites + 0.5) * np.array([edge / nxy, edge / nxy, edge / nz])
    tilt = rng.uniform(0, 0.1, n)
    az = rng.uniform(0, 2 * math.pi, n)
    dirs = np.stack([np.sin(tilt) * np.cos(az), np.sin(tilt) * np.sin(az), np.cos(tilt)], 1)
    return box, pos, dirs, _perp(rng, dirs)


def lattice_psc(n, phi=0.2, seed=1, temper=1.0):
    """PSC (the nvt_psc model) from an aligned lattice start."""
    rng = np.random.default_rng(seed)
    box, pos, dirs, pds = _lattice(rng, n, phi)
    top = ("[Types]\nP 1 PSC 1.0 1.0 1.12 0.2 90.0 10.0 3.0 0.0\n"
           f"[Molecules]\nP: {{\nparticles: 1\n}}\n[System]\nP {n}\n")
    opts = options_text(ptype=0, transmx=0.4, rotmx=30.0, temper=temper, seed=seed)
    return opts, top, config_text(box, pos, dirs, pds)


PSC_CPSC_TYPES = ("P 1 PSC 1.0 1.0 1.12 0.2 90.0 10.0 3.0 0.0\n"
                  "C 2 CPSC 1.0 1.0 1.12 0.2 120.0 10.0 3.0 0.0\n")


def psc_cpsc(n=65536, phi=0.2, seed=1, temper=1.0):
    """PSC (patch 90 deg) and CPSC (cylindrical patch 120 deg) 50/50, L=3, eps=1,
    pdis 1.12, pswitch 0.2, from an aligned lattice start (the bench melts it first).
    Particles of one type are listed together, as the [System] section requires."""
    rng = np.random.default_rng(seed)
    box, pos, dirs, pds = _lattice(rng, n, phi)
    n1 = n // 2
    top = ("[Types]\n" + PSC_CPSC_TYPES +
           "[Molecules]\nP: {\nparticles: 1\n}\nC: {\nparticles: 2\n}\n"
           f"[System]\nP {n1}\nC {n - n1}\n")
    opts = options_text(ptype=0, transmx=0.4, rotmx=30.0, temper=temper, seed=seed)
    return opts, top, config_text(box, pos, dirs, pds)


def rods_in_spheres(n_side=21, n_rods=2, L=6.0, edge=34.0, seed=1, temper=1.0):
    """A few long PSC rods among many attractive spheres (SPA on a cubic lattice of
    n_side^3 sites, minus the sites the rods overlap): the long cut-off gives 4 cells per
    edge and cell stencils of several thousand particles, so the move kernel stages its
    candidates in windows."""
    rng = np.random.default_rng(seed)
    box = np.full(3, edge)
    a = edge / n_side
    g = (np.arange(n_side) + 0.5) * a
    sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rpos = rng.uniform(0, edge, size=(n_rods, 3))
    rdir = _unit(rng, n_rods)
    keep = np.ones(len(sites), bool)
    for c, d in zip(rpos, rdir):
        r = sites - c
        r -= box * np.round(r / box)
        t = np.clip(r @ d, -L / 2, L / 2)
        dist = np.linalg.norm(r - t[:, None] * d[None, :], axis=1)
        keep &= dist > 1.05
    sph = sites[keep]
    pos = np.concatenate([rpos, sph])
    dirs = np.concatenate([rdir, _unit(rng, len(sph))])
    top = ("[Types]\n"
           f"P 1 PSC 1.0 1.0 1.12 0.2 90.0 10.0 {L} 0.0\n"
           "A 2 SPA 0.5 1.0 1.1225 0.3775\n"
           "[Molecules]\nP: {\nparticles: 1\n}\nA: {\nparticles: 2\n}\n"
           f"[System]\nP {n_rods}\nA {len(sph)}\n")
    opts = options_text(ptype=0, transmx=0.3, rotmx=20.0, temper=temper, seed=seed)
    return opts, top, config_text(box, pos, dirs, _perp(rng, dirs))


LIPID_TOP = ("[Types]\n"
             "H 1 SPN 1.0 1.0\n"
             "T 2 TPSC 1.0 1.0 1.12 0.2 90.0 10.0 2.0 0.0 180.0 90.0 10.0\n"
             "[Molecules]\nL: {\nparticles: 1\nparticles: 2\nparticles: 2\nbond1: 50.0 1.0\n}\n")


def _lipid(centre_head, u):
    """Particle centres of a straight lipid whose head sits at centre_head, tails along -u:
    bonds (50 kT, rest length 1) join the head centre to the first tail's +u end and the
    tails' facing ends."""
    return [centre_head, centre_head - 2.0 * u, centre_head - 5.0 * u]


def _lipid_texts(box, heads, axes, rng, opts):
    pos, dirs = [], []
    for h, u in zip(heads, axes):
        pos += _lipid(h, u)
        dirs += [u, u, u]
    pos, dirs = np.array(pos), np.array(dirs)
    # each particle's axis tilted by ~0.03 rad on its own: exactly collinear bonded tails sit
    # on the reference's intersection branch points (its pair energy jumps there, so the
    # energy of a chain would change under a rigid move by rounding alone)
    dirs = dirs + 0.03 * rng.normal(size=dirs.shape)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    top = LIPID_TOP + f"[System]\nL {len(heads)}\n"
    return opts, top, config_text(box, pos, dirs, _perp(rng, dirs))


def lipids_dilute(n=64, edge=14.0, seed=1, temper=1.5, chainprob=0.2):
    """n three-bead lipids (SPN head, two TPSC tails of length 2, bonds k=50, r0=1) at random,
    non-overlapping positions and orientations in a cubic box."""
    rng = np.random.default_rng(seed)
    box = np.full(3, edge)
    heads, axes, segs = [], [], []
    while len(heads) < n:
        h = rng.uniform(0, edge, 3)
        u = _unit(rng, 1)[0]
        mine = [(c, l) for c, l in zip(_lipid(h, u), (0.0, 1.0, 1.0))]
        ok = True
        for (c1, l1) in mine:
            for (c2, d2, l2) in segs:
                r = c1 - c2
                r -= box * np.round(r / box)
                if np.linalg.norm(r) > l1 + l2 + 1.05:
                    continue
                if _segdist(c2 + r, u, l1, c2[None, :], d2[None, :], np.array([l2]))[0] < 1.05:
                    ok = False
                    break
            if not ok:
                break
        if ok:
            heads.append(h)
            axes.append(u)
            segs += [(c, u, l) for c, l in mine]
    opts = options_text(ptype=0, transmx=0.3, rotmx=20.0, temper=temper, seed=seed, chainprob=chainprob,
                        chainmmx=0.3, chainrmx=15.0)
    return _lipid_texts(box, np.array(heads), np.array(axes), rng, opts)


def bilayers(n_side=50, box=(60.0, 60.0, 40.0), seed=1, temper=1.0, chainprob=0.1):
    """Lipid bilayers: 4 n_side^2 three-bead lipids (10,000 for n_side = 50) in two flat
    bilayers normal to z (centred at a quarter and three quarters of the box height), heads
    on a square lattice of spacing box_x / n_side in each leaflet, tails towards the
    bilayer middle."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, float)
    a = box[0] / n_side
    g = (np.arange(n_side) + 0.5) * a
    xy = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    heads, axes = [], []
    for zc in (0.25 * box[2], 0.75 * box[2]):
        for side in (+1.0, -1.0):
            # the lower leaflet is shifted by half a spacing and every lipid tilted by up to
            # 0.05 rad: exactly stacked, parallel tails make the reference's patch angle
            # 0/0 (perpendicular part of a vector along the axis)
            off = 0.0 if side > 0 else 0.5 * a
            for x, y in xy:
                tilt, az = rng.uniform(0.01, 0.05), rng.uniform(0, 2 * math.pi)
                u = side * np.array([math.sin(tilt) * math.cos(az), math.sin(tilt) * math.sin(az), math.cos(tilt)])
                heads.append(np.array([x + off, y + off, zc + side * 6.5]))
                axes.append(u)
    opts = options_text(ptype=0, transmx=0.3, rotmx=20.0, temper=temper, seed=seed, chainprob=chainprob,
                        chainmmx=0.3, chainrmx=15.0)
    return _lipid_texts(box, np.array(heads), np.array(axes), rng, opts)


def protein_bilayer(n_side=20, box=(30.0, 30.0, 40.0), seed=1, temper=1.0, chainprob=0.1, wlm=(1, 3)):
    """A cylindrical-patch particle (CPSC, length 2: the tails' length, one SC length per
    system) above one lipid bilayer of 2 n_side^2 three-bead lipids, with Wang-Landau weights
    over its height relative to the system centre (order 1) and its axis z component
    (order 3) -- the setting of the reference's membrane example (options wlm = 1 3).
    Returns options, top.init, config.init and the weights file (flat, alpha 0.05)."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, float)
    a = box[0] / n_side
    g = (np.arange(n_side) + 0.5) * a
    xy = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    heads, axes = [], []
    zc = 0.0                # the bilayer at z = 0, where the wrapped centre of Conf::massCenter sits
    for side in (+1.0, -1.0):
        off = 0.0 if side > 0 else 0.5 * a
        for x, y in xy:
            tilt, az = rng.uniform(0.01, 0.05), rng.uniform(0, 2 * math.pi)
            u = side * np.array([math.sin(tilt) * math.cos(az), math.sin(tilt) * math.sin(az), math.cos(tilt)])
            heads.append(np.array([x + off, y + off, zc + side * 6.5]))
            axes.append(u)
    pos, dirs = [np.array([0.5 * box[0], 0.5 * box[1], 0.3 * box[2]])], [_unit(rng, 1)[0]]
    for h, u in zip(heads, axes):
        pos += _lipid(h, u)
        dirs += [u, u, u]
    pos, dirs = np.array(pos), np.array(dirs)
    dirs = dirs + 0.03 * rng.normal(size=dirs.shape)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    top = LIPID_TOP.replace("[Molecules]\n", "P 3 CPSC 1.0 1.0 1.12 0.2 120.0 10.0 2.0 0.0\n[Molecules]\nP: {\nparticles: 3\n}\n")
    top += f"[System]\nP 1\nL {len(heads)}\n"
    opts = options_text(ptype=0, transmx=0.3, rotmx=20.0, temper=temper, seed=seed, chainprob=chainprob,
                        chainmmx=0.3, chainrmx=15.0, wlm=" ".join(str(m) for m in wlm), wlmtype=3)
    lines = ["0.05"]
    for j in range(21):
        for i in range(79):
            lines.append(f"{-19.5 + 0.5 * i:.6f} {-1.0 + 0.1 * j:.6f} 0.0 0")
    wl = "\n".join(lines) + "\n"
    return opts, top, config_text(box, pos, dirs, _perp(rng, dirs)), wl


def pt_ladders(n_ladders=8, per_ladder=8, seed=1, n_range=(500, 4000), phi_range=(0.10, 0.25), t_range=(0.8, 1.6)):
    """Parallel-tempering replicas of the PSC model with uneven sizes: n_ladders systems
    (N and packing fraction drawn uniformly), each replicated over a geometric
    temperature ladder.  Returns (texts per ladder, temperatures per ladder slot)."""
    rng = np.random.default_rng(seed)
    systems = []
    for g in range(n_ladders):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        phi = float(rng.uniform(*phi_range))
        systems.append(lattice_psc(n, phi=phi, seed=seed * 1000 + g))
    temps = list(np.geomspace(t_range[0], t_range[1], per_ladder))
    return systems, temps


def nvt_psc_grand_switch(n=1000, phi=0.1, seed=1, temper=1.0, activity=0.01, switchprob=0.1):
    """nvt_psc with its molecule grand-canonical (top.init ACTIVITY, one insert / delete move
    per sweep) and switchable to a CPSC type of the same length (patch 120 degrees, delta_mu
    1), switchprob type switch attempts per particle move."""
    opts, top, cfg = nvt_psc(n, phi=phi, seed=seed, temper=temper)
    top = top.replace("particles: 1\n", f"particles: 1 2 1.0\nACTIVITY: {activity}\n", 1)
    top = top.replace("[Molecules]", "Q 2 CPSC 1.0 1.0 1.12 0.2 120.0 10.0 3.0 0.0\n[Molecules]", 1)
    opts = opts.replace("nGrandCanon = 0", "nGrandCanon = 1").replace("switchprob = 0.0", f"switchprob = {switchprob}")
    return opts, top, cfg


WORKLOADS = {
    "npt_cpsc_spa_4000": lambda seed=1: npt_cpsc_spa(4000, seed=seed),
    "nvt_psc_1000": lambda seed=1: nvt_psc(1000, seed=seed),
    "psc_cpsc_65536": lambda seed=1: psc_cpsc(65536, seed=seed),
    "bilayer_30000": lambda seed=1: bilayers(50, seed=seed),
}
