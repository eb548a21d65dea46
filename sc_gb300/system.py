"""Python host mirror of the reference's energy / move interface, over the C ABI.

Method names follow the reference (robertvacha/SC, scOOP):
  p2p              TotalE::p2p                 scOOP/mc/totalenergycalculator.h:200-203
  one_to_all       TotalEMatrix::oneToAll(Trial)  totalenergycalculator.h:355-415
  all_to_all       TotalEMatrix::allToAll         totalenergycalculator.h:334-353
  mol2others       TotalEMatrix::mol2othersTrial  totalenergycalculator.h:453-499
  simulate         Updater::simulate              scOOP/mc/updater.cpp:45-389
  wl_*             WangLandau init / write / end  scOOP/mc/wanglandau.cpp:49-433
Every call goes to the CUDA library; a missing library raises.
"""
import ctypes as C

import numpy as np

from . import _lib as L


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class System:
    def __init__(self, handle):
        self._h = handle
        self._lib = L.load()

    @classmethod
    def open(cls, options_path, top_path, config_path):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.sc_open(str(options_path).encode(), str(top_path).encode(), str(config_path).encode(), C.byref(h)))
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

    def particles(self, first=0, count=None, out=None):
        """A ctypes array of ``sc_particle`` records (indexable, iterable, and accepted
        as is by ``set_particles``).  ``out``: an array of at least ``count`` records to
        fill instead of a new one (a caller that reads the state every step keeps one)."""
        count = self.n - first if count is None else count
        if out is not None and isinstance(out, C.Array) and out._type_ is L.Particle and len(out) >= count:
            arr = out
        else:
            arr = (L.Particle * count)()
        L.check(self._lib.sc_get_particles(self._h, first, count, arr))
        return arr

    def set_particles(self, first, parts):
        if isinstance(parts, C.Array) and parts._type_ is L.Particle:
            arr = parts
        else:
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

    def alignment_order(self):
        """Updater::alignmentOrder: sum of axis dot products over pairs closer than 1.5."""
        e = C.c_double()
        L.check(self._lib.sc_alignment_order(self._h, C.byref(e)))
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

    def pair_features(self, I, J):
        """Surrogate inputs (n x 16), WCA32 and eligibility of ordered pairs (I moved, J)."""
        I = np.ascontiguousarray(I, dtype=np.int32)
        J = np.ascontiguousarray(J, dtype=np.int32)
        n = len(I)
        X = np.zeros((n, 16), dtype=np.float32)
        W = np.zeros(n, dtype=np.float32)
        E = np.zeros(n, dtype=np.int32)
        L.check(self._lib.sc_pair_features(self._h, n, _iptr(I), _iptr(J), _fptr(X), _fptr(W), _iptr(E)))
        return X, W, E.astype(bool)

    def set_surrogate(self, sur):
        L.check(self._lib.sc_set_surrogate(self._h, sur._h if sur is not None else None))

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

    def nematic_order(self):
        """(S2, director): the largest eigenvalue of the axes' Q tensor and its eigenvector."""
        v = C.c_double()
        d = np.zeros(3)
        L.check(self._lib.sc_nematic_order(self._h, C.byref(v), _dptr(d)))
        return v.value, d

    def screen_survivors(self, targets=None, cap=None):
        """The move kernels' candidate screens over every (target, particle) pair: (i, j,
        stage_b) of the pairs that pass stage A (see sc_screen_survivors)."""
        T = None if targets is None else np.ascontiguousarray(targets, dtype=np.int32)
        nt = self.n if T is None else len(T)
        cap = cap if cap is not None else max(1024, nt * 512)
        I = np.zeros(cap, np.int32)
        J = np.zeros(cap, np.int32)
        B = np.zeros(cap, np.uint8)
        cnt = C.c_long()
        L.check(self._lib.sc_screen_survivors(self._h, nt, None if T is None else _iptr(T), cap, _iptr(I), _iptr(J),
                                              B.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(cnt)))
        k = cnt.value
        return I[:k], J[:k], B[:k]

    # --- equilibration (Updater::simulate's step adjustment, main.cpp:270-287) ----------------
    def step_sizes(self):
        st = L.StepSizes()
        L.check(self._lib.sc_get_step_sizes(self._h, C.byref(st)))
        return st

    def adjust_steps(self):
        L.check(self._lib.sc_adjust_steps(self._h))

    def equilibrate(self, nequil, adjust, params=None, **overrides):
        p = params if params is not None else self.default_run()
        for k, v in overrides.items():
            setattr(p, k, v)
        st = L.RunStats()
        L.check(self._lib.sc_equilibrate(self._h, C.byref(p), int(nequil), int(adjust), C.byref(st)))
        return st

    def tune(self, params=None, sweeps=8, **overrides):
        """sc_tune: the fastest (stencil, variant) for params' mode on the current state (which
        it leaves unchanged); later runs with variant = -1 use it.  Returns (best params,
        moves/s of every candidate)."""
        p = params if params is not None else self.default_run()
        for k, v in overrides.items():
            setattr(p, k, v)
        best = L.RunParams()
        rates = (C.c_double * 32)()
        n = C.c_int()
        L.check(self._lib.sc_tune(self._h, C.byref(p), int(sweeps), C.byref(best), rates, C.byref(n)))
        return best, [rates[k] for k in range(n.value)]

    def simulate(self, params=None, **overrides):
        p = params if params is not None else self.default_run()
        for k, v in overrides.items():
            setattr(p, k, v)
        st = L.RunStats()
        L.check(self._lib.sc_simulate(self._h, C.byref(p), C.byref(st)))
        return st

    # --- grand-canonical species (MoveCreator::muVTMove, movecreator.cpp:797-924) -------------
    def write_top_last(self, path):
        """top.last (main.cpp:313-331): top.init up to [System], then the current counts."""
        L.check(self._lib.sc_write_top_last(self._h, str(path).encode()))

    def grand_stats(self):
        """Statistics::grand of every grand-canonical species, summed over the context's runs:
        a list of sc_grand_stats records (mol_type, count, activity, chem_pot, steps, ins_acc,
        ins_rej, del_acc, del_rej, average_particles)."""
        k = C.c_int()
        L.check(self._lib.sc_grand_species(self._h, C.byref(k)))
        out = []
        for i in range(k.value):
            g = L.GrandStats()
            L.check(self._lib.sc_grand_stats_get(self._h, i, C.byref(g)))
            out.append(g)
        return out

    # --- Wang-Landau (WangLandau, scOOP/mc/wanglandau.h, wanglandau.cpp) ----------------
    def wl_load(self, path=None, text=None):
        """WangLandau::initCalc + init: weights file by path or as text."""
        if text is not None:
            L.check(self._lib.sc_wl_load_text(self._h, text.encode()))
        else:
            L.check(self._lib.sc_wl_load(self._h, str(path).encode()))

    def wl_info(self):
        i = L.WlInfo()
        L.check(self._lib.sc_wl_get_info(self._h, C.byref(i)))
        return i

    def wl_weights(self):
        """(weights, hist) of every bin, order 0 running fastest."""
        i = self.wl_info()
        nb = i.length[0] * max(1, i.length[1])
        w = np.zeros(nb)
        h = np.zeros(nb, dtype=np.int64)
        L.check(self._lib.sc_wl_get(self._h, _dptr(w), h.ctypes.data_as(C.POINTER(C.c_long))))
        return w, h

    @staticmethod
    def wl_share(walkers):
        """Walkers 1.. update walkers[0]'s weights and histogram (the reference's multiple
        walkers); run them together in a ReplicaSet with exchange_every = 0."""
        lib = L.load()
        hs = (C.c_void_p * len(walkers))(*[w._h for w in walkers])
        L.check(lib.sc_wl_share(hs, len(walkers)))

    def wl_write(self, path):
        L.check(self._lib.sc_wl_write(self._h, str(path).encode()))

    def wl_end(self, path):
        """WangLandau::endWangLandau: the final weights file."""
        L.check(self._lib.sc_wl_end(self._h, str(path).encode()))


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


class Surrogate:
    """Learned pair-energy surrogate (no counterpart in the reference): the first stage of
    delayed-acceptance moves (``simulate(delayed=1)`` after ``system.set_surrogate``)."""

    N_PARAMS = 9409

    def __init__(self, system, seed=1, capacity=0):
        self._lib = L.load()
        h = C.c_void_p()
        L.check(self._lib.sc_surrogate_create(system._h, int(seed), int(capacity), C.byref(h)))
        self._h = h

    def collect(self, system):
        total = C.c_long()
        L.check(self._lib.sc_surrogate_collect(self._h, system._h, C.byref(total)))
        return total.value

    @property
    def num_samples(self):
        v = C.c_long()
        L.check(self._lib.sc_surrogate_num_samples(self._h, C.byref(v)))
        return v.value

    def train(self, epochs, batch=8192, lr=2e-3, lr_final=0.0, warmup_steps=100, seed=1):
        p = L.TrainParams(epochs=epochs, batch=batch, lr=lr, lr_final=lr_final, warmup_steps=warmup_steps, seed=seed)
        st = L.TrainStats()
        losses = np.zeros(max(epochs, 1))
        L.check(self._lib.sc_surrogate_train(self._h, C.byref(p), _dptr(losses), C.byref(st)))
        return st, losses[:epochs]

    def evaluate(self, system):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        n = C.c_long()
        L.check(self._lib.sc_surrogate_evaluate(self._h, system._h, C.byref(a), C.byref(b), C.byref(c), C.byref(n)))
        return {"rmse": a.value, "mae": b.value, "max_abs": c.value, "pairs": n.value}

    @property
    def weights(self):
        w = np.zeros(self.N_PARAMS, dtype=np.float32)
        L.check(self._lib.sc_surrogate_get_weights(self._h, _fptr(w)))
        return w

    @weights.setter
    def weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.shape == (self.N_PARAMS,)
        L.check(self._lib.sc_surrogate_set_weights(self._h, _fptr(w)))

    def gradient(self, X, y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.N_PARAMS, dtype=np.float32)
        loss = C.c_double()
        L.check(self._lib.sc_surrogate_gradient(self._h, len(y), _fptr(X), _fptr(y), _fptr(g), C.byref(loss)))
        return g, loss.value

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(len(X), dtype=np.float32)
        L.check(self._lib.sc_surrogate_predict(self._h, len(X), _fptr(X), _fptr(out)))
        return out

    def close(self):
        if self._h:
            self._lib.sc_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
