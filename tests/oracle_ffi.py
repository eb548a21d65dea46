"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so) for the tests.

The oracle is test infrastructure: only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, always as the checker.
"""
import ctypes as C
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
                ("max_moves", C.c_long)]


class McStats(C.Structure):
    _fields_ = [(k, C.c_long) for k in ("moves", "acc_trans", "rej_trans", "acc_rot", "rej_rot", "acc_vol",
                                        "rej_vol", "acc_chain", "rej_chain")] + [
        ("energy", C.c_double), ("energy_start", C.c_double), ("seconds", C.c_double)]


class WlState(C.Structure):
    _fields_ = [("wlm", C.c_int * 2), ("len", C.c_int * 2), ("minorder", C.c_double * 2), ("dorder", C.c_double * 2),
                ("alpha", C.c_double), ("weights", C.POINTER(C.c_double)), ("hist", C.POINTER(C.c_long)),
                ("cur", C.c_long * 2), ("updates", C.c_long), ("converged", C.c_int), ("pad_", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True, capture_output=True)
        L = C.CDLL(LIB)
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
        L.or_wl_orders.argtypes = [C.POINTER(System), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_long), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
        _lib = L
    return _lib


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

    def wl_run(self, opts, wlm, minorder, dorder, length, alpha, weights, hist):
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
        rc, cur, _, _ = self.wl_orders(wlm, minorder, dorder)
        assert rc == 0
        st.cur[0], st.cur[1] = cur
        ms = McStats()
        rc = lib().or_wl_run(C.byref(self.sys), C.byref(opts), C.byref(st), C.byref(ms))
        assert rc == 0
        return w, h, st, ms

    def wl_orders(self, wlm, minorder, dorder):
        """Starting Wang-Landau bins, system centre and sysvolume (or_wl_orders)."""
        m = (C.c_int * 2)(*wlm)
        lo = (C.c_double * 2)(*minorder)
        d = (C.c_double * 2)(*dorder)
        out = (C.c_long * 2)()
        cm = (C.c_double * 3)()
        sv = C.c_double()
        rc = lib().or_wl_orders(C.byref(self.sys), m, lo, d, out, cm, C.byref(sv))
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
