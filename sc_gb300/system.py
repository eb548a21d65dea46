"""Python host mirror of the reference's energy / move interface, over the C ABI.

Method names follow the reference (robertvacha/SC, scOOP):
  p2p              TotalE::p2p                 scOOP/mc/totalenergycalculator.h:200-203
  one_to_all       TotalEMatrix::oneToAll(Trial)  totalenergycalculator.h:355-415
  all_to_all       TotalEMatrix::allToAll         totalenergycalculator.h:334-353
  mol2others       TotalEMatrix::mol2othersTrial  totalenergycalculator.h:453-499
  simulate         Updater::simulate              scOOP/mc/updater.cpp:45-389
Every call goes to the CUDA library; a missing library raises.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class System:
    def __init__(self, handle):
        self._h = handle
        self._lib = L.load()

    @classmethod
    def open(cls, options_path, top_path, config_path):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.sc_open(options_path.encode(), top_path.encode(), config_path.encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def from_text(cls, options, top, config):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.sc_open_text(options.encode("latin-1"), top.encode("latin-1"), config.encode("latin-1"),
                                 C.byref(h)))
        return cls(h)

    def close(self):
        if self._h:
            self._lib.sc_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- state ---------------------------------------------------------------------------
    @property
    def n(self):
        v = C.c_int()
        L.check(self._lib.sc_num_particles(self._h, C.byref(v)))
        return v.value

    @property
    def box(self):
        b = np.zeros(3)
        L.check(self._lib.sc_get_box(self._h, _dptr(b)))
        return b

    @box.setter
    def box(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        L.check(self._lib.sc_set_box(self._h, _dptr(b)))

    def cutoff(self):
        a, b = C.c_double(), C.c_double()
        L.check(self._lib.sc_cutoff(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def pair_param(self, t1, t2):
        p = L.PairParam()
        L.check(self._lib.sc_get_pair_param(self._h, t1, t2, C.byref(p)))
        return p

    def particles(self, first=0, count=None):
        count = self.n - first if count is None else count
        arr = (L.Particle * max(count, 1))()
        L.check(self._lib.sc_get_particles(self._h, first, count, arr))
        return arr[:count]

    def set_particles(self, first, parts):
        arr = (L.Particle * len(parts))(*parts)
        L.check(self._lib.sc_set_particles(self._h, first, len(parts), arr))

    def write_config(self, path):
        L.check(self._lib.sc_write_config(self._h, path.encode()))

    # --- energies ------------------------------------------------------------------------
    def p2p(self, i, j):
        e = C.c_double()
        L.check(self._lib.sc_pair_energy(self._h, i, j, C.byref(e)))
        return e.value

    def pair_energies(self, I, J):
        I = np.ascontiguousarray(I, dtype=np.int32)
        J = np.ascontiguousarray(J, dtype=np.int32)
        n = len(I)
        E = np.zeros(n)
        V = np.zeros(n, dtype=np.uint32)
        D = np.zeros(n)
        L.check(self._lib.sc_pair_energies(self._h, n, _iptr(I), _iptr(J), _dptr(E),
                                           V.ctypes.data_as(C.POINTER(C.c_uint)), _dptr(D)))
        return E, V, D

    def one_to_all(self, targets):
        T = np.ascontiguousarray(np.atleast_1d(targets), dtype=np.int32)
        out = np.zeros(len(T))
        L.check(self._lib.sc_one_to_all(self._h, len(T), _iptr(T), _dptr(out)))
        return out

    def all_to_all(self):
        e = C.c_double()
        L.check(self._lib.sc_all_to_all(self._h, C.byref(e)))
        return e.value

    def mol2others(self, first, size):
        e = C.c_double()
        L.check(self._lib.sc_mol_to_others(self._h, first, size, C.byref(e)))
        return e.value

    def trial_displace(self, target, dr):
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        a, b = C.c_double(), C.c_double()
        L.check(self._lib.sc_trial_displace(self._h, target, _dptr(dr), C.byref(a), C.byref(b)))
        return a.value, b.value

    def trial_rotate(self, target, angle, axis, positive):
        ax = np.ascontiguousarray(axis, dtype=np.float64)
        a, b = C.c_double(), C.c_double()
        st = L.Particle()
        L.check(self._lib.sc_trial_rotate(self._h, target, float(angle), _dptr(ax), int(positive), C.byref(a),
                                          C.byref(b), C.byref(st)))
        return a.value, b.value, st

    def accept_trial(self):
        L.check(self._lib.sc_accept_trial(self._h))

    def trial_volume(self, psch):
        e = C.c_double()
        L.check(self._lib.sc_trial_volume(self._h, float(psch), C.byref(e)))
        return e.value

    # --- move loop -----------------------------------------------------------------------
    def default_run(self):
        p = L.RunParams()
        L.check(self._lib.sc_default_run(self._h, C.byref(p)))
        return p

    def simulate(self, params=None, **overrides):
        p = params if params is not None else self.default_run()
        for k, v in overrides.items():
            setattr(p, k, v)
        st = L.RunStats()
        L.check(self._lib.sc_simulate(self._h, C.byref(p), C.byref(st)))
        return st


class ReplicaSet:
    """Replicas moved together on one GPU, with parallel-tempering exchanges.

    The reference runs one replica per MPI rank (MoveCreator::replicaExchangeMove,
    scOOP/mc/movecreator.cpp:552-795); here every replica's moves run in the same
    kernels.  `ladder[k]` groups replicas into independent temperature ladders.
    """

    def __init__(self, systems, temperatures, ladder=None):
        self._lib = L.load()
        self.systems = list(systems)
        n = len(self.systems)
        hs = (C.c_void_p * n)(*[s._h for s in self.systems])
        T = np.ascontiguousarray(temperatures, dtype=np.float64)
        lad = None if ladder is None else np.ascontiguousarray(ladder, dtype=np.int32)
        h = C.c_void_p()
        L.check(self._lib.sc_replicas_create(hs, n, _dptr(T), None if lad is None else _iptr(lad), C.byref(h)))
        self._h = h

    def run(self, nsweeps, exchange_every=0, seed=1, params=None, **overrides):
        p = params if params is not None else self.systems[0].default_run()
        p.nsweeps = nsweeps
        p.seed = seed
        for k, v in overrides.items():
            setattr(p, k, v)
        n = len(self.systems)
        st = L.RunStats()
        T = np.zeros(n)
        E = np.zeros(n)
        tried = (C.c_long * n)()
        acc = (C.c_long * n)()
        L.check(self._lib.sc_replicas_run(self._h, C.byref(p), int(exchange_every), C.byref(st), _dptr(T), _dptr(E),
                                          tried, acc))
        return st, T, E, np.array(tried[:]), np.array(acc[:])

    def close(self):
        if self._h:
            self._lib.sc_replicas_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
