"""ctypes binding of the C ABI declared in include/sc_gb300.h (libscgpu.so).

There is no fallback: if the CUDA library is missing or fails to load, every
call raises.  Build it with ``python -c "import __graft_entry__ as g; g.build()"``
or ``python sc_gb300/build.py``.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libscgpu.so")

SC_OK = 0
ERRORS = {-1: "SC_ERR_ARG", -2: "SC_ERR_IO", -3: "SC_ERR_PARSE", -4: "SC_ERR_CUDA", -5: "SC_ERR_RANGE",
          -6: "SC_ERR_STATE", -7: "SC_ERR_UNSUPPORTED", -8: "SC_ERR_DEVICE"}


class ScError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class StepSizes(C.Structure):
    _fields_ = [("trans", C.c_double * 40), ("rot_cos", C.c_double * 40), ("chain_trans", C.c_double * 8),
                ("chain_rot_cos", C.c_double * 8), ("edge", C.c_double), ("adjustments", C.c_long)] + [
        (k, C.c_long * 40) for k in ("acc_trans", "rej_trans", "acc_rot", "rej_rot")] + [
        (k, C.c_long * 8) for k in ("acc_chain_trans", "rej_chain_trans", "acc_chain_rot", "rej_chain_rot")] + [
        ("acc_edge", C.c_long), ("rej_edge", C.c_long)]


class PairParam(C.Structure):
    _fields_ = [("geotype", C.c_int * 2), ("exclude", C.c_int), ("kind", C.c_int),
                ("sigma", C.c_double), ("epsilon", C.c_double), ("A", C.c_double), ("B", C.c_double),
                ("pdis", C.c_double), ("pswitch", C.c_double), ("pswitchINV", C.c_double),
                ("pcangl", C.c_double * 4), ("pcanglsw", C.c_double * 4),
                ("rcut", C.c_double), ("rcutSq", C.c_double), ("rcutwca", C.c_double), ("rcutwcaSq", C.c_double),
                ("pcoshalfi", C.c_double * 4), ("psinhalfi", C.c_double * 4),
                ("csecpatchrot", C.c_double * 2), ("ssecpatchrot", C.c_double * 2), ("volume", C.c_double),
                ("len", C.c_double * 2), ("half_len", C.c_double * 2), ("chiral_cos", C.c_double * 2),
                ("chiral_sin", C.c_double * 2), ("parallel", C.c_double)]


class Particle(C.Structure):
    _fields_ = [("pos", C.c_double * 3), ("dir", C.c_double * 3), ("patchdir", (C.c_double * 3) * 2),
                ("patchsides", (C.c_double * 3) * 4), ("chdir", (C.c_double * 3) * 2), ("type", C.c_int),
                ("molType", C.c_int)]


class RunParams(C.Structure):
    _fields_ = [("nsweeps", C.c_long), ("seed", C.c_ulonglong), ("temper", C.c_double), ("press", C.c_double),
                ("ptype", C.c_int), ("volume_every", C.c_int), ("transmx", C.c_double), ("rot_angle", C.c_double),
                ("edge_mx", C.c_double), ("chainprob", C.c_double), ("chainmmx", C.c_double),
                ("chain_angle", C.c_double), ("check_every", C.c_int), ("time_phases", C.c_int),
                ("stencil", C.c_int), ("delayed", C.c_int), ("variant", C.c_int), ("flow_wait_polls", C.c_int),
                ("grand_every", C.c_int), ("sweep_offset", C.c_long), ("switchprob", C.c_double)]


class RunStats(C.Structure):
    _fields_ = [(k, C.c_long) for k in ("sweeps", "moves", "acc_trans", "rej_trans", "acc_rot", "rej_rot",
                                        "acc_vol", "rej_vol", "vol_constrained", "acc_chain", "rej_chain",
                                        "pairs_tested", "pairs_evaluated")] + [
        (k, C.c_double) for k in ("energy", "energy_check", "max_drift", "seconds", "phase_seconds")] + [
        ("phase_launches", C.c_long), ("launches", C.c_long),
        ("da_stage1_rejected", C.c_long), ("da_stage2_tried", C.c_long), ("da_stage2_rejected", C.c_long),
        ("da_err_rms", C.c_double), ("da_err_mean", C.c_double)] + [
        (k, C.c_long) for k in ("acc_insert", "rej_insert", "acc_delete", "rej_delete", "particles", "acc_switch",
                                "rej_switch")]


class GrandStats(C.Structure):
    _fields_ = [("mol_type", C.c_int), ("type", C.c_int), ("count", C.c_int), ("pad_", C.c_int),
                ("activity", C.c_double), ("chem_pot", C.c_double)] + [
        (k, C.c_long) for k in ("steps", "ins_acc", "ins_rej", "del_acc", "del_rej")] + [
        ("average_particles", C.c_double)]


class TrainParams(C.Structure):
    _fields_ = [("epochs", C.c_int), ("batch", C.c_int), ("lr", C.c_double), ("lr_final", C.c_double),
                ("warmup_steps", C.c_int), ("pad_", C.c_int), ("seed", C.c_ulonglong)]


class TrainStats(C.Structure):
    _fields_ = [("steps", C.c_long), ("samples", C.c_long), ("loss_first", C.c_double), ("loss_last", C.c_double),
                ("seconds", C.c_double)]


class WlInfo(C.Structure):
    _fields_ = [("dim", C.c_int), ("wlm", C.c_int * 2), ("length", C.c_int * 2), ("converged", C.c_int),
                ("minorder", C.c_double * 2), ("dorder", C.c_double * 2), ("alpha", C.c_double),
                ("currorder", C.c_long * 2), ("updates", C.c_long), ("syscm", C.c_double * 3)]


# (name, restype, argtypes) for every entry point of include/sc_gb300.h
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_F = C.POINTER(C.c_float)
SIGNATURES = [
    ("sc_last_error", C.c_char_p, []),
    ("sc_version", C.c_char_p, []),
    ("sc_open", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(_P)]),
    ("sc_open_text", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(_P)]),
    ("sc_close", C.c_int, [_P]),
    ("sc_set_device", C.c_int, [_P, C.c_int]),
    ("sc_num_particles", C.c_int, [_P, _I]),
    ("sc_get_box", C.c_int, [_P, _D]),
    ("sc_set_box", C.c_int, [_P, _D]),
    ("sc_cutoff", C.c_int, [_P, _D, _D]),
    ("sc_get_pair_param", C.c_int, [_P, C.c_int, C.c_int, C.POINTER(PairParam)]),
    ("sc_get_particles", C.c_int, [_P, C.c_int, C.c_int, C.POINTER(Particle)]),
    ("sc_set_particles", C.c_int, [_P, C.c_int, C.c_int, C.POINTER(Particle)]),
    ("sc_write_config", C.c_int, [_P, C.c_char_p]),
    ("sc_pair_energy", C.c_int, [_P, C.c_int, C.c_int, _D]),
    ("sc_pair_energies", C.c_int, [_P, C.c_int, _I, _I, _D, C.POINTER(C.c_uint), _D]),
    ("sc_one_to_all", C.c_int, [_P, C.c_int, _I, _D]),
    ("sc_one_to_all_noalloc", C.c_int, [_P, C.c_int, _I, _D]),
    ("sc_all_to_all", C.c_int, [_P, _D]),
    ("sc_alignment_order", C.c_int, [_P, _D]),
    ("sc_mol_to_others", C.c_int, [_P, C.c_int, C.c_int, _D]),
    ("sc_trial_displace", C.c_int, [_P, C.c_int, _D, _D, _D]),
    ("sc_trial_rotate", C.c_int, [_P, C.c_int, C.c_double, _D, C.c_int, _D, _D, C.POINTER(Particle)]),
    ("sc_accept_trial", C.c_int, [_P]),
    ("sc_trial_volume", C.c_int, [_P, C.c_double, _D]),
    ("sc_default_run", C.c_int, [_P, C.POINTER(RunParams)]),
    ("sc_simulate", C.c_int, [_P, C.POINTER(RunParams), C.POINTER(RunStats)]),
    ("sc_grand_species", C.c_int, [_P, _I]),
    ("sc_grand_stats_get", C.c_int, [_P, C.c_int, C.POINTER(GrandStats)]),
    ("sc_write_top_last", C.c_int, [_P, C.c_char_p]),
    ("sc_nematic_order", C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("sc_get_step_sizes", C.c_int, [_P, C.c_void_p]),
    ("sc_adjust_steps", C.c_int, [_P]),
    ("sc_equilibrate", C.c_int, [_P, C.POINTER(RunParams), C.c_long, C.c_long, C.POINTER(RunStats)]),
    ("sc_tune", C.c_int, [_P, C.POINTER(RunParams), C.c_int, C.POINTER(RunParams), C.POINTER(C.c_double),
                          C.POINTER(C.c_int)]),
    ("sc_screen_survivors", C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.c_long, C.POINTER(C.c_int),
                                      C.POINTER(C.c_int), C.POINTER(C.c_ubyte), C.POINTER(C.c_long)]),
    ("sc_fp64_rates", C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(C.c_double)]),
    ("sc_wl_load", C.c_int, [_P, C.c_char_p]),
    ("sc_wl_load_text", C.c_int, [_P, C.c_char_p]),
    ("sc_wl_get_info", C.c_int, [_P, C.POINTER(WlInfo)]),
    ("sc_wl_share", C.c_int, [C.POINTER(_P), C.c_int]),
    ("sc_wl_get", C.c_int, [_P, _D, C.POINTER(C.c_long)]),
    ("sc_wl_write", C.c_int, [_P, C.c_char_p]),
    ("sc_wl_end", C.c_int, [_P, C.c_char_p]),
    ("sc_replicas_create", C.c_int, [C.POINTER(_P), C.c_int, _D, _I, C.POINTER(_P)]),
    ("sc_replicas_run", C.c_int, [_P, C.POINTER(RunParams), C.c_int, C.POINTER(RunStats), _D, _D,
                                  C.POINTER(C.c_long), C.POINTER(C.c_long)]),
    ("sc_replicas_destroy", C.c_int, [_P]),
    ("sc_surrogate_create", C.c_int, [_P, C.c_ulonglong, C.c_long, C.POINTER(_P)]),
    ("sc_surrogate_destroy", C.c_int, [_P]),
    ("sc_surrogate_collect", C.c_int, [_P, _P, C.POINTER(C.c_long)]),
    ("sc_surrogate_num_samples", C.c_int, [_P, C.POINTER(C.c_long)]),
    ("sc_surrogate_train", C.c_int, [_P, C.POINTER(TrainParams), _D, C.POINTER(TrainStats)]),
    ("sc_surrogate_evaluate", C.c_int, [_P, _P, _D, _D, _D, C.POINTER(C.c_long)]),
    ("sc_surrogate_get_weights", C.c_int, [_P, _F]),
    ("sc_surrogate_set_weights", C.c_int, [_P, _F]),
    ("sc_surrogate_gradient", C.c_int, [_P, C.c_int, _F, _F, _F, _D]),
    ("sc_surrogate_predict", C.c_int, [_P, C.c_int, _F, _F]),
    ("sc_pair_features", C.c_int, [_P, C.c_int, _I, _I, _F, _F, _I]),
    ("sc_set_surrogate", C.c_int, [_P, _P]),
]

_lib = None


def load():
    """Loads libscgpu.so; raises if it is not built (there is no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (python sc_gb300/build.py)")
        lib = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(rc):
    if rc != SC_OK:
        raise ScError(rc, load().sc_last_error().decode(errors="replace"))
    return rc
