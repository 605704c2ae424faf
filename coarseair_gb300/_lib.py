"""ctypes bindings of the C ABI in include/cair_gpu.h (the library libcair_gpu.so built in-tree).

The product path always goes through this library; if it is missing or no GPU is present the
calls raise.  There is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcair_gpu.so")
CAIR_MAX_PES = 64
CAIR_ABI_VERSION = 6
CAIR_STATIC_QUEUE_MAX_TRAJ = 16384

STATUS = {0: "CAIR_OK", 1: "CAIR_EINVAL", 2: "CAIR_ECUDA", 3: "CAIR_ETIMEOUT", 4: "CAIR_ENONFINITE",
          5: "CAIR_EUNSUPPORTED"}


class PesDesc(C.Structure):
    _fields_ = [("model", C.c_int32), ("ncoef", C.c_int32), ("coef", C.POINTER(C.c_double)),
                ("a", C.c_double), ("ab", C.c_double), ("ra", C.c_double), ("rb", C.c_double),
                ("eref", C.c_double), ("totdiss", C.c_double)]


class SystemDesc(C.Structure):
    _fields_ = [("abi_version", C.c_int32), ("natoms", C.c_int32), ("npes", C.c_int32),
                ("diat_model", C.c_int32), ("mass", C.c_double * 4), ("tpq", C.POINTER(C.c_double)),
                ("pes", PesDesc * CAIR_MAX_PES),
                ("dt0", C.c_double), ("eps", C.c_double), ("relax", C.c_double), ("rmax", C.c_double),
                ("tmax", C.c_double), ("ham_abs_tol", C.c_double),
                ("nsteps", C.c_int32), ("inc_step", C.c_int32), ("ncall", C.c_int32), ("nquad", C.c_int32),
                ("rsmal", C.c_double), ("rcent", C.c_double), ("rfact", C.c_double), ("tthresau", C.c_double)]


class MolState(C.Structure):
    _fields_ = [("ipair", C.c_int32), ("itype", C.c_int32), ("eint", C.c_double), ("angmom", C.c_double),
                ("viba", C.c_double)]


class TrajPoint(C.Structure):
    _fields_ = [("mol", MolState * 2), ("b", C.c_double), ("xkin", C.c_double), ("vrel", C.c_double * 3),
                ("nmol", C.c_int32), ("pad", C.c_int32)]


TRAJ_POINT_DTYPE = np.dtype([("ipair0", "i4"), ("itype0", "i4"), ("eint0", "f8"), ("angmom0", "f8"),
                             ("viba0", "f8"), ("ipair1", "i4"), ("itype1", "i4"), ("eint1", "f8"),
                             ("angmom1", "f8"), ("viba1", "f8"), ("b", "f8"), ("xkin", "f8"),
                             ("vrel", "f8", (3,)), ("nmol", "i4"), ("pad", "i4")])

class StatsParams(C.Structure):
    _fields_ = [("qn_max", C.c_int32), ("ncond", C.c_int32), ("iskip", C.c_int32 * 5),
                ("pres_even_odd", C.c_int32 * 5), ("ham_abs_tol", C.c_double), ("xmu", C.c_double)]


STATS_COUNT_DTYPE = np.dtype([("run", "i4"), ("ring", "i4"), ("code", "i8"), ("count", "i8")])
STATS_MAX_RINGS = 64
FINAL_STATE_DTYPE = np.dtype([("run", "i4"), ("fin", "i4", 5), ("ini", "i4", 5), ("nrings", "i4"), ("count", "i8"),
                              ("nrows", "i8"), ("cross", "f8"), ("cross_sd", "f8"), ("rate", "f8"),
                              ("rate_sd", "f8")])

TUNE_POINT_DTYPE = np.dtype([("block", "i4"), ("per_sm", "i4"), ("ms", "f8"), ("attempts_per_s", "f8")])
SUR_SAMPLE_DTYPE = np.dtype([("R", "f8", (3,)), ("e", "f4"), ("g", "f4", (3,))])
SUR_NINV = 10


class SurConsts(C.Structure):
    _fields_ = [("mu", C.c_float * SUR_NINV), ("isd", C.c_float * SUR_NINV), ("fmin", C.c_float * SUR_NINV),
                ("fmax", C.c_float * SUR_NINV), ("sigma_d", C.c_float), ("gate_ev", C.c_float),
                ("gate_dmin", C.c_float)]


LEVEL_DTYPE = np.dtype([("vqn", "i4"), ("jqn", "i4"), ("eint", "f8"), ("egam", "f8"), ("rmin", "f8"),
                        ("rmax", "f8"), ("vmin", "f8"), ("vmax", "f8"), ("tau", "f8"), ("ri", "f8"), ("ro", "f8")])
ITEM_DTYPE = np.dtype([("ilevel", "i4"), ("ipes", "i4"), ("first", "i8"), ("ntraj", "i8"), ("seed", "i8"),
                       ("ttra", "f8"), ("bmax", "f8"), ("dinit", "f8"), ("ilevel2", "i4"), ("b_mode", "i4"),
                       ("bmin", "f8"), ("skip", "i8")])
RESULT_DTYPE = np.dtype([("idx", "i8"), ("item", "i4"), ("ipes", "i4"), ("status", "i4"), ("iste", "i4"),
                         ("irej", "i4"), ("pad", "i4"),
                         ("bmax", "f8"), ("b", "f8"), ("j_i", "f8"), ("v_i", "f8"), ("arr_i", "f8"),
                         ("j_f", "f8"), ("v_f", "f8"), ("arr_f", "f8"), ("t", "f8"), ("dH", "f8"),
                         ("j2_i", "f8"), ("v2_i", "f8"), ("j2_f", "f8"), ("v2_f", "f8")])

# (name, restype, argtypes) of every entry point declared in include/cair_gpu.h
_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_L = C.POINTER(C.c_int64)
SIGNATURES = [
    ("cair_create", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(SystemDesc)]),
    ("cair_destroy", None, [_P]),
    ("cair_last_error", C.c_char_p, [_P]),
    ("cair_dims", C.c_int, [_P, _I, _I, _I]),
    ("cair_get_tpq", C.c_int, [_P, _D]),
    ("cair_pes_eval", C.c_int, [_P, C.c_int64, _I, _D, _D, _D, _D, _D]),
    ("cair_rhs", C.c_int, [_P, C.c_int64, _I, _D, _D]),
    ("cair_hamiltonian", C.c_int, [_P, C.c_int64, _I, _D, _D, _D]),
    ("cair_bs_steps", C.c_int, [_P, C.c_int64, _I, _D, _D, _D, _D, C.c_int32]),
    ("cair_integrate", C.c_int, [_P, C.c_int64, _I, _D, _D, _D, _D, _D, _D, _D, _I, _I, _I, C.c_int64]),
    ("cair_integrate_dev", C.c_int, [_P, C.c_int64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_int64, _P]),
    ("cair_find_state", C.c_int, [_P, C.c_int64, _D, C.POINTER(TrajPoint)]),
    ("cair_apply_transformation", C.c_int, [_P, C.c_int64, _D, _D]),
    ("cair_sample_ics", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, _D, _D, _D, _D, _D, _I]),
    ("cair_sample_ics_dev", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("cair_run_queue", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, C.c_int64, _P]),
    ("cair_run_queue_dev", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, C.c_int64, _P, _P, _P]),
    ("cair_queue_workspace_bytes", C.c_int64, [C.c_int64]),
    ("cair_run_queue_static_dev", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, C.c_int64, _P, _P]),
    ("cair_flop_model", C.c_int, [_P, C.c_int32, _D, _D, _D, _D]),
    ("cair_last_counters", C.c_int, [_P, _L]),
    ("cair_fp64_peak_probe", C.c_int, [_P, _D]),
    ("cair_statistics", C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, _P, C.POINTER(StatsParams), _P, C.c_int64, _L]),
    ("cair_statistics_dev", C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, _P, C.POINTER(StatsParams), _P, C.c_int64, _L,
                                      _P]),
    ("cair_statistics_items", C.c_int, [_P, C.c_int32, C.c_int64, _P, C.POINTER(StatsParams), _P, _P]),
    ("cair_statistics_items_dev", C.c_int, [_P, C.c_int32, C.c_int64, _P, C.POINTER(StatsParams), _P, _P, _P]),
    ("cair_statistics_counts", C.c_int, [_P, C.c_int32, _P, _P, _P, _P, C.c_int64, _P, C.POINTER(StatsParams), _P,
                                         C.c_int64, _L, _P]),
    ("cair_statistics_counts_dev", C.c_int, [_P, C.c_int32, _P, _P, _P, _P, C.c_int64, _P, C.POINTER(StatsParams),
                                             _P, C.c_int64, _L, _P, _P]),
    ("cair_statistics_finish", C.c_int, [C.c_int32, _P, _P, _P, _P, C.POINTER(StatsParams), C.c_int64, _P, _P, _P,
                                         C.c_int64, _L, C.c_char_p, C.c_int32]),
    ("cair_format_rows", C.c_int, [_P, C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_char_p, C.c_int64, _L]),
    ("cair_write_trajectories", C.c_int, [C.c_char_p, _P, C.c_int64, C.c_int64, C.c_int32, C.c_double, _L]),
    ("cair_write_trajectories_bin", C.c_int, [C.c_char_p, _P, C.c_int64, C.c_int64, C.c_int32, C.c_double]),
    ("cair_merge_trajectories", C.c_int, [C.c_int32, C.POINTER(C.c_char_p), C.c_char_p, _L]),
    ("cair_queue_graph_create", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, C.c_int64, _P, _P,
                                          C.POINTER(C.c_void_p)]),
    ("cair_queue_graph_launch", C.c_int, [_P, _P, _P]),
    ("cair_queue_graph_destroy", None, [_P]),
    ("cair_set_integrate_timing", C.c_int, [_P, C.c_int32]),
    ("cair_integrate_timings", C.c_int, [_P, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_int32)]),
    ("cair_sur_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int32]),
    ("cair_sur_destroy", None, [_P]),
    ("cair_sur_last_error", C.c_char_p, [_P]),
    ("cair_sur_nparam", C.c_int, []),
    ("cair_sur_set_consts", C.c_int, [_P, C.POINTER(SurConsts)]),
    ("cair_sur_get_consts", C.c_int, [_P, C.POINTER(SurConsts)]),
    ("cair_sur_set_params", C.c_int, [_P, C.c_int32, C.POINTER(C.c_float)]),
    ("cair_sur_get_params", C.c_int, [_P, C.c_int32, C.POINTER(C.c_float)]),
    ("cair_sur_eval_dev", C.c_int, [_P, C.c_int64, _P, _P, _P, _P, _P, _P, _P]),
    ("cair_sur_grad_dev", C.c_int, [_P, C.c_int32, C.c_int64, _P, _P, C.c_float, C.c_float, _P]),
    ("cair_sur_adam_dev", C.c_int, [_P, C.c_int32, C.c_float, _P]),
    ("cair_sur_get_grad", C.c_int, [_P, C.c_int32, C.POINTER(C.c_float)]),
    ("cair_sur_take_loss", C.c_int, [_P, _D, _P]),
    ("cair_sur_counters", C.c_int, [_P, _L, C.c_int32]),
    ("cair_sur_targets_dev", C.c_int, [_P, C.c_int64, _P, _P, _P]),
    ("cair_sur_attach", C.c_int, [_P, _P]),
    ("cair_record_samples", C.c_int, [_P, _P, C.c_int64, C.c_int32, C.c_double]),
    ("cair_set_warp_timeline", C.c_int, [_P, _P, C.c_int64]),
    ("cair_warp_timeline_count", C.c_int64, [_P]),
    ("cair_set_launch_shape", C.c_int, [_P, C.c_int32, C.c_int32]),
    ("cair_get_launch_shape", C.c_int, [_P, _I, _I]),
    ("cair_autotune", C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, C.c_int64, C.c_int64, _P, C.c_int32, _I]),
    ("cair_recorded_samples", C.c_int64, [_P]),
    ("cair_set_integrator_mode", C.c_int, [_P, C.c_int32]),
    ("cair_get_integrator_mode", C.c_int32, [_P]),
    ("cair_last_integrator", C.c_int32, [_P]),
    ("cair_set_tail_handoff", C.c_int, [_P, C.c_int64]),
    ("cair_last_handoffs", C.c_int64, [_P]),
    ("cair_internal_warp_eval", C.c_int, [_P, C.c_int64, _P, _P, _P, _P, _P]),
]
INTEGRATOR_THREAD, INTEGRATOR_WARP, INTEGRATOR_AUTO = 0, 1, 2

_lib = None


def load(path=LIB_PATH):
    """Load libcair_gpu.so and declare its entry points.  Raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libcair_gpu.so is not built (run __graft_entry__.build()): %s" % path)
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a):
    return a.ctypes.data_as(_D) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_I) if a is not None else None
