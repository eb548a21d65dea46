"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so) for the tests.

The oracle is test infrastructure: only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, always to check or time against, never as a product path.
"""
import ctypes as C
import math
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
MAXT = 40
GEOTYPES = {"SCN": 10, "SCA": 11, "PSC": 12, "CPSC": 13, "CHPSC": 14, "CHCPSC": 15, "TPSC": 16, "TCPSC": 17,
            "TCHPSC": 18, "TCHCPSC": 19, "SP": 30, "SPN": 30, "SPA": 31}


class Vec(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class Param(C.Structure):
    _fields_ = [("geotype", C.c_int * 2), ("exclude", C.c_int), ("pad_", C.c_int),
                ("sigma", C.c_double), ("epsilon", C.c_double), ("A", C.c_double), ("B", C.c_double),
                ("pdis", C.c_double), ("pswitch", C.c_double), ("pswitchINV", C.c_double),
                ("pcangl", C.c_double * 4), ("pcanglsw", C.c_double * 4),
                ("rcut", C.c_double), ("rcutSq", C.c_double), ("rcutwca", C.c_double), ("rcutwcaSq", C.c_double),
                ("pcoshalfi", C.c_double * 4), ("psinhalfi", C.c_double * 4),
                ("csecpatchrot", C.c_double * 2), ("ssecpatchrot", C.c_double * 2), ("volume", C.c_double),
                ("len", C.c_double * 2), ("half_len", C.c_double * 2), ("chiral_cos", C.c_double * 2),
                ("chiral_sin", C.c_double * 2), ("parallel", C.c_double)]


class TypeIn(C.Structure):
    _fields_ = [("type", C.c_int), ("geotype", C.c_int), ("nfields", C.c_int), ("pad_", C.c_int),
                ("param", C.c_double * 12)]


class Particle(C.Structure):
    _fields_ = [("pos", Vec), ("dir", Vec), ("pd", Vec * 2), ("ps", Vec * 4), ("ch", Vec * 2),
                ("type", C.c_int), ("molType", C.c_int)]


class MolType(C.Structure):
    _fields_ = [("size", C.c_int), ("first", C.c_int), ("count", C.c_int), ("pad_", C.c_int)] + [
        (k, C.c_double) for k in ("bond1c", "bond1eq", "bond2c", "bond2eq", "bonddc", "bonddeq", "bondhc",
                                  "bondheq", "angle1c", "angle1eq", "angle2c", "angle2eq")]


class System(C.Structure):
    _fields_ = [("n", C.c_int), ("nmol", C.c_int), ("p", C.POINTER(Particle)), ("mols", C.POINTER(MolType)),
                ("params", C.POINTER(Param)), ("box", C.c_double * 3), ("sqmaxcut", C.c_double)]


class McOpts(C.Structure):
    _fields_ = [("nsweeps", C.c_long), ("seed", C.c_long), ("temper", C.c_double), ("press", C.c_double),
                ("shave", C.c_double), ("chainprob", C.c_double), ("transmx", C.c_double),
                ("rot_angle", C.c_double), ("edge_mx", C.c_double), ("chainmmx", C.c_double),
                ("chainr_angle", C.c_double), ("ptype", C.c_int), ("pairlist_update", C.c_int),
                ("max_moves", C.c_long), ("energy_matrix", C.c_int), ("pad_", C.c_int),
                ("switchprob", C.c_double), ("switch_other", C.POINTER(C.c_int)), ("switch_dmu", C.POINTER(C.c_int)),
                ("switched", C.POINTER(C.c_int)), ("grand_every", C.c_int), ("n_gc", C.c_int), ("gc_cap", C.c_int),
                ("pad2_", C.c_int), ("gc_moltype", C.POINTER(C.c_int)), ("gc_type", C.POINTER(C.c_int)),
                ("gc_chempot", C.POINTER(C.c_double))]


class McStats(C.Structure):
    _fields_ = [(k, C.c_long) for k in ("moves", "acc_trans", "rej_trans", "acc_rot", "rej_rot", "acc_vol",
                                        "rej_vol", "acc_chain", "rej_chain")] + [
        ("energy", C.c_double), ("energy_start", C.c_double), ("seconds", C.c_double),
        ("acc_switch", C.c_long), ("rej_switch", C.c_long), ("acc_insert", C.c_long), ("rej_insert", C.c_long),
        ("acc_delete", C.c_long), ("rej_delete", C.c_long)]


class WlState(C.Structure):
    _fields_ = [("wlm", C.c_int * 2), ("len", C.c_int * 2), ("minorder", C.c_double * 2), ("dorder", C.c_double * 2),
                ("alpha", C.c_double), ("weights", C.POINTER(C.c_double)), ("hist", C.POINTER(C.c_long)),
                ("cur", C.c_long * 2), ("updates", C.c_long), ("converged", C.c_int), ("wlmtype", C.c_int)]


LIB_FAST = os.path.join(ROOT, "oracle", "_build", "liboracle_fast.so")
_libs = {}


def lib(fast=False):
    """The oracle library; fast=True: its -Ofast build (CPU timing legs only)."""
    path = LIB_FAST if fast else LIB
    if path not in _libs:
        if not os.path.exists(path):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True, capture_output=True)
        _libs[path] = _bind(C.CDLL(path))
    return _libs[path]


def _bind(L):
    if True:
        L.or_pair_energy.restype = C.c_double
        L.or_pair_energy.argtypes = [C.POINTER(System), C.c_int, C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_double)]
        L.or_one_to_all.restype = C.c_double
        L.or_one_to_all.argtypes = [C.POINTER(System), C.c_int]
        L.or_all_to_all.restype = C.c_double
        L.or_all_to_all.argtypes = [C.POINTER(System)]
        L.or_mol2others.restype = C.c_double
        L.or_mol2others.argtypes = [C.POINTER(System), C.c_int, C.c_int]
        L.or_derive_params.restype = C.c_int
        L.or_derive_params.argtypes = [C.POINTER(TypeIn), C.c_int, C.c_void_p, C.POINTER(Param),
                                       C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_particle_init.argtypes = [C.POINTER(Particle), C.POINTER(Param)]
        L.or_psc_rotate.argtypes = [C.POINTER(Particle), C.c_int, C.c_double, Vec, C.c_int]
        L.or_mc_run.restype = C.c_int
        L.or_mc_run.argtypes = [C.POINTER(System), C.POINTER(McOpts), C.POINTER(McStats)]
        L.or_wl_run.restype = C.c_int
        L.or_wl_run.argtypes = [C.POINTER(System), C.POINTER(McOpts), C.POINTER(WlState), C.POINTER(McStats)]
        L.or_wl_orders.restype = C.c_int
        L.or_wl_orders.argtypes = [C.POINTER(System), C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_long), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
        L.or_nematic.restype = C.c_int
        L.or_nematic.argtypes = [C.POINTER(System), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_pair_energies.restype = None
        L.or_pair_energies.argtypes = [C.POINTER(System), C.c_long, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_double), C.POINTER(C.c_uint), C.POINTER(C.c_double)]
        L.or_prefilter_pairs.restype = None
        L.or_prefilter_pairs.argtypes = [C.POINTER(System), C.c_int, C.POINTER(C.c_int), C.c_long,
                                         C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_long)]
        L.or_mc_open.restype = C.c_void_p
        L.or_mc_open.argtypes = [C.POINTER(System), C.POINTER(McOpts)]
        L.or_mc_advance.restype = C.c_int
        L.or_mc_advance.argtypes = [C.c_void_p, C.c_long, C.POINTER(McStats)]
        L.or_mc_sweeps.restype = C.c_int
        L.or_mc_sweeps.argtypes = [C.c_void_p, C.c_long, C.POINTER(McStats)]
        L.or_mc_energy.restype = C.c_double
        L.or_mc_energy.argtypes = [C.c_void_p]
        L.or_mc_setup_seconds.restype = C.c_double
        L.or_mc_setup_seconds.argtypes = [C.c_void_p]
        L.or_mc_close.argtypes = [C.c_void_p]
    return L


def vec(a):
    return Vec(float(a[0]), float(a[1]), float(a[2]))


def params_from_ref(ref):
    table = (Param * (MAXT * MAXT))()
    scalar = ("sigma", "epsilon", "A", "B", "pdis", "pswitch", "pswitchINV", "rcut", "rcutSq", "rcutwca",
              "rcutwcaSq", "volume", "parallel")
    arrays = ("pcangl", "pcanglsw", "pcoshalfi", "psinhalfi", "csecpatchrot", "ssecpatchrot", "len", "half_len",
              "chiral_cos", "chiral_sin")
    for e in ref["ia_params"]:
        p = table[e["t1"] * MAXT + e["t2"]]
        p.geotype[0], p.geotype[1] = e["geotype"]
        p.exclude = e["exclude"]
        for k in scalar:
            setattr(p, k, float(e[k]))
        for k in arrays:
            arr = getattr(p, k)
            for q, v in enumerate(e[k]):
                arr[q] = float(v)
    return table


def particle_from_ref(d):
    p = Particle()
    p.pos, p.dir = vec(d["pos"]), vec(d["dir"])
    p.pd[0], p.pd[1] = vec(d["pd0"]), vec(d["pd1"])
    for k in range(4):
        p.ps[k] = vec(d[f"ps{k}"])
    p.ch[0], p.ch[1] = vec(d["ch0"]), vec(d["ch1"])
    p.type, p.molType = d["type"], d["molType"]
    return p


def mols_from_ref(ref):
    ms = (MolType * max(1, len(ref["molecules"])))()
    for k, m in enumerate(ref["molecules"]):
        ms[k].size, ms[k].first, ms[k].count = m["size"], m["first"], m["count"]
        for key in ("bond1", "bond2", "bondd", "bondh", "angle1", "angle2"):
            setattr(ms[k], key + "c", float(m[key][0]))
            setattr(ms[k], key + "eq", float(m[key][1]))
    return ms


class OracleSystem:
    """Keeps the ctypes buffers alive together with the System struct."""

    def __init__(self, ref, particles=None):
        self.params = params_from_ref(ref)
        self.mols = mols_from_ref(ref)
        plist = particles if particles is not None else ref["particles"]
        self.parts = (Particle * len(plist))(*[particle_from_ref(d) for d in plist])
        self.sys = System()
        self.sys.n = len(plist)
        self.sys.nmol = len(ref["molecules"])
        self.sys.p = C.cast(self.parts, C.POINTER(Particle))
        self.sys.mols = C.cast(self.mols, C.POINTER(MolType))
        self.sys.params = C.cast(self.params, C.POINTER(Param))
        for k in range(3):
            self.sys.box[k] = float(ref["box"][k])
        self.sys.sqmaxcut = float(ref["sqmaxcut"])

    def set_state(self, parts, box):
        """Takes a configuration from the GPU path (sc_particle records and box edges), e.g.
        after device sweeps, so that the oracle evaluates that state."""
        for k, q in enumerate(parts):
            o = self.parts[k]
            o.pos, o.dir = vec(q.pos), vec(q.dir)
            for m in range(2):
                o.pd[m], o.ch[m] = vec(q.patchdir[m]), vec(q.chdir[m])
            for m in range(4):
                o.ps[m] = vec(q.patchsides[m])
            assert o.type == q.type
        for k in range(3):
            self.sys.box[k] = float(box[k])

    def pair(self, i, j):
        bits = C.c_uint(0)
        dsq = C.c_double(0)
        e = lib().or_pair_energy(C.byref(self.sys), i, j, C.byref(bits), C.byref(dsq))
        return e, bits.value, dsq.value

    def one_to_all(self, i):
        return lib().or_one_to_all(C.byref(self.sys), i)

    def all_to_all(self):
        return lib().or_all_to_all(C.byref(self.sys))

    def mol2others(self, first, size):
        return lib().or_mol2others(C.byref(self.sys), first, size)

    def wl_run(self, opts, wlm, minorder, dorder, length, alpha, weights, hist, wlmtype=-1):
        """Sequential Wang-Landau run (or_wl_run); returns (weights, hist, state, stats)."""
        w = np.ascontiguousarray(weights, dtype=np.float64).copy()
        h = np.ascontiguousarray(hist, dtype=np.int64).copy()
        st = WlState()
        st.wlm[0], st.wlm[1] = wlm
        st.len[0], st.len[1] = length
        st.minorder[0], st.minorder[1] = minorder
        st.dorder[0], st.dorder[1] = dorder
        st.alpha = alpha
        st.weights = w.ctypes.data_as(C.POINTER(C.c_double))
        st.hist = h.ctypes.data_as(C.POINTER(C.c_long))
        st.wlmtype = wlmtype
        rc, cur, _, _ = self.wl_orders(wlm, minorder, dorder, wlmtype)
        assert rc == 0
        st.cur[0], st.cur[1] = cur
        ms = McStats()
        rc = lib().or_wl_run(C.byref(self.sys), C.byref(opts), C.byref(st), C.byref(ms))
        assert rc == 0
        return w, h, st, ms

    def wl_orders(self, wlm, minorder, dorder, wlmtype=-1):
        """Starting Wang-Landau bins, system centre and sysvolume (or_wl_orders; wlmtype: the
        particle type of the mesh and contact orders)."""
        m = (C.c_int * 2)(*wlm)
        lo = (C.c_double * 2)(*minorder)
        d = (C.c_double * 2)(*dorder)
        out = (C.c_long * 2)()
        cm = (C.c_double * 3)()
        sv = C.c_double()
        rc = lib().or_wl_orders(C.byref(self.sys), m, int(wlmtype), lo, d, out, cm, C.byref(sv))
        return rc, [out[0], out[1]], [cm[0], cm[1], cm[2]], sv.value


def parse_types(top_text):
    """The [Types] section of a top.init as TypeIn records (fields = numbers after EPSILON SIGMA)."""
    out, excl = [], np.zeros((MAXT, MAXT), np.uint8)
    key = None
    for raw in top_text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if line.startswith("["):
            key = line[1:].split("]")[0].strip().upper()
            continue
        if key == "TYPES":
            tok = line.split()
            name, num, geo = tok[0], int(tok[1]), tok[2]
            vals = [float(x) for x in tok[3:]]
            t = TypeIn()
            t.type, t.geotype, t.nfields = num, GEOTYPES[geo], len(vals) - 2
            for k, v in enumerate(vals[:12]):
                t.param[k] = v
            out.append(t)
        elif key == "EXCLUDE":
            nums = [int(x) for x in line.split()]
            for a, b in zip(nums[::2], nums[1::2]):
                excl[a, b] = excl[b, a] = 1
    return out, excl


# --- the oracle's own set-up from the reference's three inputs ---------------------------------
# Restates Sim::readOptions (scOOP/structures/sim.h:123-406, unit conversions :359-366),
# Inicializer::initTop / initConfig (scOOP/mc/inicializer.cpp:16-298: [Types], [Molecules],
# [System], the box line, per-particle lines, usePBC, makeMoleculeWhole) and partVecInit
# (scOOP/structures/Conf.cpp:97-102) without the GPU library, so that a CPU baseline sets up
# its system from the same texts the GPU path reads.

PIH = 1.57079632679489661923132169163975


def parse_options(text):
    d = {}
    for raw in text.splitlines():
        line = raw.split("#", 1)[0]
        if "=" not in line:
            continue
        k, v = line.split("=", 1)
        d[k.strip()] = v.strip()
    return d


def molecules(top):
    """[Molecules] definitions (name, particle types, bond constants) in definition order (the
    molType index) and the [System] entries (name, count) in order."""
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
                cur = {"name": line.split(":")[0].strip(), "types": [], "bonds": {}}
                defs.append(cur)
            elif line.startswith("}"):
                cur = None
            elif cur is not None and ":" in line:
                k, v = line.split(":", 1)
                k = k.strip().lower()
                if k == "particles":     # TYPE [SWITCHTYPE DELTA_MU] (inicializer.cpp:955-985)
                    w = v.split()
                    cur["types"].append(int(w[0]))
                    cur.setdefault("switch", []).append((int(w[1]), float(w[2])) if len(w) >= 3 else (-1, 0.0))
                elif k == "activity":    # inicializer.cpp:1087-1096
                    cur["activity"] = float(v.split()[0])
                else:
                    cur["bonds"][k] = [float(x) for x in v.split()[:2]]
        elif key == "SYSTEM":
            name, cnt = line.split()[:2]
            order.append((name, int(cnt)))
    return defs, order


def _normalise(v):
    t = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    if t != 0.0:
        t = 1.0 / t
        return [v[0] * t, v[1] * t, v[2] * t]
    return v


class TextSystem:
    """An or_system (with its ctypes buffers) and McOpts set up from options / top.init /
    config.init texts by the oracle alone."""

    def __init__(self, options, top, config):
        opts = parse_options(options)
        types, excl = parse_types(top)
        arr = (TypeIn * len(types))(*types)
        self.params = (Param * (MAXT * MAXT))()
        sq, mc = C.c_double(), C.c_double()
        if lib().or_derive_params(arr, len(types), excl.ctypes.data, self.params, C.byref(sq), C.byref(mc)) != 0:
            raise ValueError("oracle: top.init rejected")
        defs, order = molecules(top)
        ptypes, pmol, psw = [], [], []
        first = {}
        for name, cnt in order:
            m = next(k for k, d in enumerate(defs) if d["name"] == name)
            first.setdefault(m, (len(ptypes), cnt))
            for _ in range(cnt):
                for q, ty in enumerate(defs[m]["types"]):
                    ptypes.append(ty)
                    pmol.append(m)
                    psw.append(defs[m].get("switch", [(-1, 0.0)] * len(defs[m]["types"]))[q])
        self.mols = (MolType * max(1, len(defs)))()
        for k, d in enumerate(defs):
            ms = self.mols[k]
            ms.size = len(d["types"])
            ms.first, ms.count = first.get(k, (0, 0))
            for b in ("bond1", "bond2", "bondd", "bondh", "angle1", "angle2"):
                c, eq = d["bonds"].get(b, [-1.0, -1.0])
                setattr(ms, b + "c", c)
                setattr(ms, b + "eq", eq)
        lines = [l.split("#", 1)[0].strip() for l in config.splitlines()]
        lines = [l for l in lines if l]
        box = [float(x) for x in lines[0].replace("x", " ").split()[-3:]]
        n = len(ptypes)
        if len(lines) - 1 < n:
            raise ValueError("config.init: fewer particle lines than [System] declares")
        # grand-canonical species (single particles with an ACTIVITY): free slots for insertions
        gcs = [k for k, d in enumerate(defs) if "activity" in d and len(d["types"]) == 1]
        self.cap = n + (max(256, 2 * n) if gcs else 0)
        self.parts = (Particle * max(1, self.cap))()
        # per particle: the other type of its switch pair (-1: none), delta_mu as the move's int
        self.switch_other = (C.c_int * max(1, n))(*([t for t, _ in psw] + [0] * (n == 0)))
        self.switch_dmu = (C.c_int * max(1, n))(*([int(d) for _, d in psw] + [0] * (n == 0)))
        self.switched = (C.c_int * max(1, n))()
        for i in range(n):
            f = [float(x) for x in lines[1 + i].split()[:9]]
            pos = [f[0] / box[0], f[1] / box[1], f[2] / box[2]]
            for k in range(3):                      # Cuboid::usePBC
                while pos[k] < 0.0:
                    pos[k] += 1.0
                while pos[k] > 1.0:
                    pos[k] -= 1.0
            d = _normalise(f[3:6])
            pd = f[6:9]
            dp = pd[0] * d[0] + pd[1] * d[1] + pd[2] * d[2]
            pd = _normalise([pd[0] - dp * d[0], pd[1] - dp * d[1], pd[2] - dp * d[2]])
            p = self.parts[i]
            p.pos, p.dir, p.pd[0] = vec(pos), vec(d), vec(pd)
            p.type, p.molType = ptypes[i], pmol[i]
            # the switched column: the particle starts in its switch type (inicializer.cpp:226-236)
            fields = lines[1 + i].split()
            if len(fields) >= 10 and int(fields[9]) and psw[i][0] >= 0:
                self.switched[i] = 1
                p.type = psw[i][0]
                self.switch_other[i] = ptypes[i]
        for k, d in enumerate(defs):                # Conf::makeMoleculeWhole
            size = len(d["types"])
            if size <= 1:
                continue
            f0, cnt = first.get(k, (0, 0))
            for s in range(f0, f0 + size * cnt, size):
                for q in range(s + 1, s + size):
                    a, b = self.parts[q].pos, self.parts[q - 1].pos
                    r = [(a.x - b.x), (a.y - b.y), (a.z - b.z)]
                    r = [(x - round(x)) for x in r]
                    self.parts[q].pos = Vec(b.x + r[0], b.y + r[1], b.z + r[2])
        for i in range(n):
            t = self.parts[i].type
            lib().or_particle_init(C.byref(self.parts[i]), C.byref(self.params[t * MAXT + t]))
        self.gc_moltype = (C.c_int * max(1, len(gcs)))(*(gcs or [0]))
        self.gc_type = (C.c_int * max(1, len(gcs)))(*([defs[k]["types"][0] for k in gcs] or [0]))
        self.gc_chempot = (C.c_double * max(1, len(gcs)))(
            *([math.log(defs[k]["activity"] * 6.022137e23 * 1e-24) for k in gcs] or [0.0]))
        self.sys = System()
        self.sys.n, self.sys.nmol = n, len(defs)
        self.sys.p = C.cast(self.parts, C.POINTER(Particle))
        self.sys.mols = C.cast(self.mols, C.POINTER(MolType))
        self.sys.params = C.cast(self.params, C.POINTER(Param))
        for k in range(3):
            self.sys.box[k] = box[k]
        self.sys.sqmaxcut = sq.value
        o = McOpts()
        o.seed = int(opts.get("seed", "1"))
        o.temper = float(opts.get("temper", "1"))
        o.press = float(opts.get("press", "0"))
        o.shave = float(opts.get("shave", "0"))
        o.transmx = 2.0 * float(opts.get("transmx", "0"))
        o.rot_angle = float(opts.get("rotmx", "0")) / 180.0 * PIH * 0.5
        o.edge_mx = 2.0 * float(opts.get("edge_mx", "0"))
        o.chainprob = float(opts.get("chainprob", "0"))
        o.chainmmx = 2.0 * float(opts.get("chainmmx", "0"))
        o.chainr_angle = float(opts.get("chainrmx", "0")) / 180.0 * PIH
        o.ptype = int(opts.get("ptype", "0").split()[0])
        o.pairlist_update = int(opts.get("pairlist_update", "0"))
        o.nsweeps = int(opts.get("nsweeps", "0"))
        o.switchprob = float(opts.get("switchprob", "0"))
        o.switch_other, o.switch_dmu, o.switched = self.switch_other, self.switch_dmu, self.switched
        o.grand_every = int(opts.get("nGrandCanon", "0")) if gcs else 0
        o.n_gc, o.gc_cap = len(gcs), self.cap
        o.gc_moltype, o.gc_type, o.gc_chempot = self.gc_moltype, self.gc_type, self.gc_chempot
        self.opts = o

    def all_to_all(self):
        return lib().or_all_to_all(C.byref(self.sys))

    def one_to_all(self, t):
        return lib().or_one_to_all(C.byref(self.sys), int(t))

    def nematic(self):
        """(S2, director) of the oracle (or_nematic)."""
        v = C.c_double()
        d = (C.c_double * 3)()
        lib().or_nematic(C.byref(self.sys), C.byref(v), d)
        return v.value, np.array(d[:])

    def set_state(self, parts, box):
        """Takes a configuration from the GPU path (sc_particle records and box edges)."""
        OracleSystem.set_state(self, parts, box)

    def pair_energies(self, I, J):
        I = np.ascontiguousarray(I, dtype=np.int32)
        J = np.ascontiguousarray(J, dtype=np.int32)
        n = len(I)
        E = np.zeros(n)
        B = np.zeros(n, np.uint32)
        D = np.zeros(n)
        lib().or_pair_energies(C.byref(self.sys), n, I.ctypes.data_as(C.POINTER(C.c_int)),
                               J.ctypes.data_as(C.POINTER(C.c_int)), E.ctypes.data_as(C.POINTER(C.c_double)),
                               B.ctypes.data_as(C.POINTER(C.c_uint)), D.ctypes.data_as(C.POINTER(C.c_double)))
        return E, B, D

    def prefilter_pairs(self, targets=None):
        """Ordered pairs (i, j) PairE's prefilter admits (distance or bond)."""
        T = None if targets is None else np.ascontiguousarray(targets, dtype=np.int32)
        nt = self.sys.n if T is None else len(T)
        tp = None if T is None else T.ctypes.data_as(C.POINTER(C.c_int))
        cnt = C.c_long()
        lib().or_prefilter_pairs(C.byref(self.sys), nt, tp, 0, None, None, C.byref(cnt))
        I = np.zeros(max(1, cnt.value), np.int32)
        J = np.zeros(max(1, cnt.value), np.int32)
        lib().or_prefilter_pairs(C.byref(self.sys), nt, tp, cnt.value, I.ctypes.data_as(C.POINTER(C.c_int)),
                                 J.ctypes.data_as(C.POINTER(C.c_int)), C.byref(cnt))
        return I[:cnt.value], J[:cnt.value]


class McRun:
    """The oracle's sequential loop on a TextSystem, opened once (set-up outside any timing)
    and advanced by `moves` at a time."""

    def __init__(self, ts, seed=None, energy_matrix=True, fast=False):
        self.ts = ts
        self.L = lib(fast)
        o = ts.opts
        if seed is not None:
            o.seed = seed
        o.energy_matrix = 1 if energy_matrix else 0
        self.h = self.L.or_mc_open(C.byref(ts.sys), C.byref(o))
        if not self.h:
            raise ValueError("oracle: loop refused (empty system without grand-canonical species, a ptype "
                             "outside 0..5, or grand-canonical moves with switching)")
        self.stats = McStats()

    @property
    def setup_seconds(self):
        return self.L.or_mc_setup_seconds(self.h)

    @property
    def energy(self):
        return self.L.or_mc_energy(self.h)

    def advance(self, moves):
        if self.L.or_mc_advance(self.h, int(moves), C.byref(self.stats)) != 0:
            raise RuntimeError("oracle: or_mc_advance failed")
        return self.stats

    def sweeps(self, n):
        if self.L.or_mc_sweeps(self.h, int(n), C.byref(self.stats)) != 0:
            raise RuntimeError("oracle: or_mc_sweeps failed")
        return self.stats

    @property
    def n(self):
        """The particle count now (grand-canonical moves change it)."""
        return self.ts.sys.n

    def close(self):
        if self.h:
            self.L.or_mc_close(self.h)
            self.h = None
