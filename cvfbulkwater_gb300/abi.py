"""ctypes binding of include/cvf.h (the C ABI of the GB300 engine).

This is the binding a Python caller of the engine uses; the struct layouts mirror cvf.h field
for field. ``lib()`` loads the in-tree library built by ``cvfbulkwater_gb300.build`` and raises
if it is absent -- the engine has no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcvf_gb300.so")


class CvfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cvf error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("L", C.c_int), ("T", C.c_float), ("P", C.c_float), ("seed", C.c_longlong),
                ("R_cutoff", C.c_float), ("start", C.c_int), ("flag_chessboard", C.c_int),
                ("replica", C.c_uint), ("device", C.c_int), ("sample_capacity", C.c_int)]


class Obs(C.Structure):
    _fields_ = [("n_hb2", C.c_longlong), ("n_sigma", C.c_longlong), ("r_cell", C.c_double),
                ("volume", C.c_double), ("e_vdw", C.c_double), ("n_hb", C.c_double),
                ("energy", C.c_double), ("enthalpy", C.c_double), ("v_total", C.c_double),
                ("m", C.c_double)]


class CStats(C.Structure):
    _fields_ = [("largest", C.c_longlong), ("second", C.c_longlong), ("n_percolating", C.c_longlong),
                ("n_clusters", C.c_longlong), ("sum_size", C.c_longlong), ("sum_size2", C.c_longlong),
                ("sum_size2_wrap32", C.c_longlong), ("mean", C.c_double), ("variance", C.c_double),
                ("mean_ref", C.c_float), ("variance_ref", C.c_float)]


class Sample(C.Structure):
    _fields_ = [("n_hb2", C.c_longlong), ("n_sigma", C.c_longlong), ("r_cell", C.c_double),
                ("volume", C.c_double)]


class State(C.Structure):
    _fields_ = [("r_cell", C.c_double), ("volume", C.c_double), ("e_vdw", C.c_double),
                ("counters", C.c_uint * 4)]


class RunStats(C.Structure):
    _fields_ = [("L", C.c_int), ("P", C.c_double), ("T", C.c_double), ("mean", C.c_double * 6),
                ("var", C.c_double * 6), ("n", C.c_longlong)]


_POINT = ("T", "energy", "energy_err", "enthalpy", "enthalpy_err", "volume", "volume_err", "density",
          "density_err", "nhb", "nhb_err", "ncoop", "ncoop_err", "rcell", "rcell_err", "cp_fluc", "kt_fluc")
_POINT_SI = ("T_K", "density", "density_err", "enthalpy", "enthalpy_err", "energy", "energy_err", "cp_fluc",
             "cp_fluc_err", "nhb", "nhb_err", "ncoop", "ncoop_err")


class IsobarPoint(C.Structure):
    _fields_ = [(n, C.c_double) for n in _POINT]


class IsobarPointSI(C.Structure):
    _fields_ = [(n, C.c_double) for n in _POINT_SI]


class Input(C.Structure):
    _fields_ = [("P", C.c_float), ("T", C.c_float), ("seed", C.c_longlong), ("metropolis_steps", C.c_int),
                ("cluster_steps", C.c_int), ("equilibrium_steps", C.c_int), ("sampling_steps", C.c_int),
                ("sampling_interval", C.c_int), ("R_cutoff", C.c_float), ("flag_config", C.c_int),
                ("flag_distances", C.c_int), ("flag_correlation", C.c_int), ("flag_chessboard", C.c_int),
                ("device_id", C.c_int), ("L", C.c_int)]


_lib = None


def lib():
    """Load the engine library (raises FileNotFoundError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(f"{LIB_PATH} not built: run cvfbulkwater_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    I, LL, D = C.c_int, C.c_longlong, C.c_double
    sig = {
        "cvf_last_error_string": (C.c_char_p, []),
        "cvf_version": (C.c_char_p, []),
        "cvf_create": (I, [C.POINTER(Params), C.POINTER(P)]),
        "cvf_batch_create": (I, [C.POINTER(Params), I, C.POINTER(P)]),
        "cvf_destroy": (I, [P]),
        "cvf_num_replicas": (I, [P]),
        "cvf_set_config": (I, [P, I, P, LL]),
        "cvf_get_config": (I, [P, I, P, LL]),
        "cvf_set_arms": (I, [P, I, P, P, LL]),
        "cvf_get_arms": (I, [P, I, P, P, LL]),
        "cvf_set_distances": (I, [P, I, P, P, I]),
        "cvf_get_distances": (I, [P, I, P, P, I, C.POINTER(I)]),
        "cvf_run_steps": (I, [P, I, I, I]),
        "cvf_batch_run": (I, [P, I, I, I]),
        "cvf_run_sampled": (I, [P, I, I, I, I]),
        "cvf_synchronize": (I, [P]),
        "cvf_observables": (I, [P, I, C.POINTER(Obs)]),
        "cvf_cluster_stats": (I, [P, I, C.POINTER(CStats)]),
        "cvf_get_labels": (I, [P, I, P, LL]),
        "cvf_sample_count": (I, [P, I, C.POINTER(LL)]),
        "cvf_get_samples": (I, [P, I, P, LL, C.POINTER(LL)]),
        "cvf_sample_stream": (I, [P, I, P, LL, C.POINTER(LL)]),
        "cvf_get_cstats_stream": (I, [P, I, P, LL, C.POINTER(LL)]),
        "cvf_clear_samples": (I, [P]),
        "cvf_sample_observables": (I, [P, I, C.POINTER(Sample), C.POINTER(Obs)]),
        "cvf_get_state": (I, [P, I, C.POINTER(State)]),
        "cvf_set_state": (I, [P, I, C.POINTER(State)]),
        "cvf_get_thresholds": (I, [P, I, P]),
        "cvf_get_stream": (I, [P, C.POINTER(P)]),
        "cvf_autotune": (I, [P, C.POINTER(I)]),
        "cvf_set_sweep_tile": (I, [P, I, C.POINTER(I)]),
        "cvf_set_launch_mode": (I, [P, I]),
        "cvf_get_launch_mode": (I, [P, C.POINTER(I)]),
        "cvf_set_io_mode": (I, [P, I]),
        "cvf_get_io_mode": (I, [P, C.POINTER(I)]),
        "cvf_profile_launch": (I, [P, I, I]),
        "cvf_cluster_stats_noalloc": (I, [P, I, P, P]),
        "cvf_set_wait_limits": (I, [P, C.c_longlong, C.c_longlong]),
        "cvf_packed_size": (I, [P, I, C.POINTER(LL)]),
        "cvf_set_row_tile": (I, [P, I]),
        "cvf_get_tuning": (I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
        "cvf_get_packed": (I, [P, I, P, LL]),
        "cvf_set_packed": (I, [P, I, P, LL]),
        "cvf_read_input_data": (I, [C.c_char_p, C.POINTER(Input)]),
        "cvf_read_config_file": (I, [C.c_char_p, P, LL]),
        "cvf_write_config_file": (I, [C.c_char_p, P, LL]),
        "cvf_write_distances_file": (I, [C.c_char_p, I, P, P, I]),
        "cvf_read_distances_file": (I, [C.c_char_p, I, P, P, I, C.POINTER(I)]),
        "cvf_format_data_line": (I, [C.c_char_p, I, I, C.POINTER(Obs)]),
        "cvf_format_cluster_line": (I, [C.c_char_p, I, I, C.POINTER(CStats)]),
        "cvf_set_replica_groups": (I, [P, I]),
        "cvf_get_replica_groups": (I, [P, C.POINTER(I)]),
        "cvf_h2d_create": (I, [I, P, P, P, LL, P, P, I, I, D, I, C.POINTER(P)]),
        "cvf_h2d_info": (I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(D), C.POINTER(D), C.POINTER(D), C.POINTER(D), P]),
        "cvf_h2d_reweight": (I, [P, D, D, P, C.POINTER(D), C.POINTER(D)]),
        "cvf_h2d_mixed": (I, [P, D, P, P, C.POINTER(D)]),
        "cvf_h2d_mixed_batch": (I, [P, P, I, P, P, P]),
        "cvf_h2d_ising": (I, [P, P, I, D, P]),
        "cvf_h2d_scan": (I, [P, P, I, P, I, P, I, D, P, P, P]),
        "cvf_h2d_set_constants": (I, [P, P]),
        "cvf_h2d_destroy": (I, [P]),
        "cvf_set_correlation": (I, [P, I]),
        "cvf_set_cluster_algorithm": (I, [P, I]),
        "cvf_wolff_stats": (I, [P, I, P]),
        "cvf_set_wolff_counter": (I, [P, I, C.c_ulonglong]),
        "cvf_get_correlation": (I, [P, I, P, P, I, C.POINTER(I)]),
        "cvf_run_statistics": (I, [P, C.POINTER(RunStats), I]),
        "cvf_isobar_point_from_stats": (I, [C.POINTER(RunStats), C.POINTER(IsobarPoint)]),
        "cvf_isobar_point_to_si": (I, [C.POINTER(IsobarPoint), D, C.POINTER(IsobarPointSI)]),
        "cvf_alpha_p_derivative": (I, [P, P, P, P, I, P, P, P, C.POINTER(I)]),
        "cvf_cp_derivative": (I, [P, P, P, P, I, P, P, P, C.POINTER(I)]),
        "cvf_kt_derivative": (I, [P, P, P, P, I, P, P]),
        "cvf_reweight_forward": (I, [I, P, P, LL, P, I, P, I, D, D, P, P, I, P]),
        "cvf_reweight_adjoint": (I, [I, P, P, LL, P, I, P, D, P, P, I, P, P]),
    }
    for name, (res, args) in sig.items():
        if not hasattr(L, name):
            continue
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int):
    if rc != 0:
        msg = lib().cvf_last_error_string()
        raise CvfError(rc, msg.decode() if msg else "")
