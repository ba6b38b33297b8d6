"""ctypes binding of libmlff_gb300.so (include/mlff_gb300.h).

The library is the only compute path: if it is missing or no CUDA device is
present, every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Optional

from . import _build

MAX_LAYERS = 8

OK = 0
ERR_INVALID = 1
ERR_CAPACITY = 2
ERR_CUDA = 3
ERR_TIMEOUT = 4
ERR_UNSUPPORTED = 5
ERR_BOX = 6
ERR_ROW = 7
ERR_WORKSPACE = 8

PATH_PLAIN_FP32 = 0
PATH_TUNED_TC = 1
PATH_TUNED_FP32 = 2
PATH_TRAIN = 3
PATH_TRAIN_FORCES = 4

PATHS = {"plain": PATH_PLAIN_FP32, "fp32": PATH_PLAIN_FP32, "plain_fp32": PATH_PLAIN_FP32,
         "fp16x3": PATH_TUNED_TC, "tc": PATH_TUNED_TC, "tuned": PATH_TUNED_TC,
         "tuned_fp32": PATH_TUNED_FP32}

ERROR_NAMES = {ERR_INVALID: "invalid argument", ERR_CAPACITY: "edge capacity exceeded",
               ERR_CUDA: "CUDA error", ERR_TIMEOUT: "device wait timed out",
               ERR_UNSUPPORTED: "unsupported model shape", ERR_BOX: "invalid periodic box",
               ERR_ROW: "too many neighbours in one row", ERR_WORKSPACE: "workspace too small"}

EXPORTS = ["mlff_version", "mlff_last_error_string", "mlff_packed_weights_size", "mlff_pack_weights",
           "mlff_workspace_size", "mlff_build_neighbors", "mlff_copy_neighbors", "mlff_energy_forces",
           "mlff_read_status", "mlff_clear_status", "mlff_verlet_steps", "mlff_langevin_steps", "mlff_npt_steps",
           "mlff_langevin_ase_steps",
           "mlff_md_energy_stats",
           "mlff_profile_begin",
           "mlff_profile_end", "mlff_radius_graph_noalloc", "mlff_param_grads", "mlff_param_grads_forces",
           "mlff_debug_stall_test", "mlff_painn_message_workspace_size", "mlff_painn_message",
           "mlff_painn_message_backward", "mlff_painn_update_workspace_size", "mlff_painn_update",
           "mlff_painn_update_backward", "mlff_force_stats_workspace_size", "mlff_force_stats",
           "mlff_autotune", "mlff_autotune_query", "mlff_autotune_set", "mlff_autotune_query_shape",
           "mlff_autotune_set_shape", "mlff_autotune_reset"]

PROFILE_KINDS = ["neighbors", "edge_fwd", "edge_bwd", "update_fwd", "update_bwd", "readout", "forces",
                 "plain_gemm", "plain_edge", "other", "md", "edge_bwd_q"]


class Dims(ctypes.Structure):
    _fields_ = [("hidden", ctypes.c_int32), ("n_rbf", ctypes.c_int32), ("n_layers", ctypes.c_int32),
                ("n_species", ctypes.c_int32), ("cutoff", ctypes.c_float)]


_P = ctypes.c_void_p
_PL = _P * MAX_LAYERS


class Params(ctypes.Structure):
    _fields_ = [("embedding", _P), ("rbf_centers", _P), ("rbf_widths", _P),
                ("filter_w1", _PL), ("filter_b1", _PL), ("filter_w2", _PL), ("filter_b2", _PL),
                ("mixing", _PL), ("update_w1", _PL), ("update_b1", _PL), ("update_w2", _PL),
                ("update_b2", _PL), ("head_w1", _P), ("head_b1", _P), ("head_w2", _P),
                ("head_b2", _P), ("head_w3", _P), ("head_b3", _P)]


class Grads(ctypes.Structure):
    """mlff_grads: gradient output pointers, same layout as Params."""
    _fields_ = Params._fields_


class System(ctypes.Structure):
    _fields_ = [("n_atoms", ctypes.c_int32), ("n_mol", ctypes.c_int32), ("pos", _P), ("Z", _P),
                ("mol_ptr", _P), ("box", _P), ("pbc", _P)]


class Outputs(ctypes.Structure):
    _fields_ = [("energy", _P), ("forces", _P), ("virial", _P), ("atom_energy", _P)]


class MDState(ctypes.Structure):
    _fields_ = [("pos", _P), ("vel", _P), ("inv_mass", _P), ("forces", _P), ("energy", _P),
                ("kinetic", _P), ("energy_trace", _P), ("kinetic_trace", _P), ("step_counter", _P)]


class NPTState(ctypes.Structure):
    _fields_ = [("box", _P), ("box32", _P), ("zeta", _P), ("eta", _P), ("xi", _P), ("virial", _P)]


class MLFFError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, 'error')} (code {code}): {msg}")
        self.code = code


class CapacityError(MLFFError):
    def __init__(self, code, msg, needed):
        super().__init__(code, msg)
        self.needed = needed


_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load the shared library (building it first if it is absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError(f"{path} is missing; run mlff_gb300._build.build()")
            _build.build()
        lib = ctypes.CDLL(path)
        i32, i64, sz = ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t
        lib.mlff_version.restype = ctypes.c_int
        lib.mlff_last_error_string.restype = ctypes.c_char_p
        lib.mlff_packed_weights_size.restype = sz
        lib.mlff_packed_weights_size.argtypes = [ctypes.POINTER(Dims)]
        lib.mlff_pack_weights.restype = ctypes.c_int
        lib.mlff_pack_weights.argtypes = [ctypes.POINTER(Dims), ctypes.POINTER(Params), _P, sz, _P]
        lib.mlff_workspace_size.restype = sz
        lib.mlff_workspace_size.argtypes = [ctypes.POINTER(Dims), i32, i32, i64, i32]
        lib.mlff_build_neighbors.restype = ctypes.c_int
        lib.mlff_build_neighbors.argtypes = [ctypes.POINTER(Dims), ctypes.POINTER(System), i64, _P, sz, _P]
        lib.mlff_copy_neighbors.restype = ctypes.c_int
        lib.mlff_copy_neighbors.argtypes = [_P, i32, i32, i64, i32, _P, _P, _P]
        lib.mlff_energy_forces.restype = ctypes.c_int
        lib.mlff_energy_forces.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, i32,
                                           ctypes.POINTER(Outputs), _P, sz, _P]
        lib.mlff_read_status.restype = ctypes.c_int
        lib.mlff_read_status.argtypes = [_P, ctypes.POINTER(i32), ctypes.POINTER(i64), ctypes.POINTER(i32), _P]
        lib.mlff_clear_status.restype = ctypes.c_int
        lib.mlff_clear_status.argtypes = [_P, _P]
        lib.mlff_verlet_steps.restype = ctypes.c_int
        lib.mlff_verlet_steps.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, i32,
                                          ctypes.POINTER(MDState), ctypes.c_double, i32, _P, sz, _P]
        lib.mlff_langevin_steps.restype = ctypes.c_int
        lib.mlff_langevin_steps.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, i32,
                                            ctypes.POINTER(MDState), ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_uint64, i32, _P, sz, _P]
        lib.mlff_langevin_ase_steps.restype = ctypes.c_int
        lib.mlff_langevin_ase_steps.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, i32,
                                                ctypes.POINTER(MDState), ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_uint64, i32, i32, _P, sz, _P]
        lib.mlff_npt_steps.restype = ctypes.c_int
        lib.mlff_npt_steps.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, i32,
                                       ctypes.POINTER(MDState), ctypes.POINTER(NPTState), ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, i32, _P,
                                       sz, _P]
        lib.mlff_md_energy_stats.restype = ctypes.c_int
        lib.mlff_md_energy_stats.argtypes = [_P, _P, i32, i32, _P, ctypes.c_double, _P, _P]
        lib.mlff_profile_begin.restype = ctypes.c_int
        lib.mlff_profile_end.restype = ctypes.c_int
        lib.mlff_profile_end.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(i64), i32]
        lib.mlff_param_grads.restype = ctypes.c_int
        lib.mlff_param_grads.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, _P,
                                         ctypes.POINTER(Grads), ctypes.POINTER(Outputs), _P, sz, _P]
        lib.mlff_param_grads_forces.restype = ctypes.c_int
        lib.mlff_param_grads_forces.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, _P, _P,
                                                ctypes.POINTER(Grads), _P, sz, _P]
        lib.mlff_painn_message_workspace_size.restype = sz
        lib.mlff_painn_message_workspace_size.argtypes = [i32, i32, i64, i32]
        lib.mlff_painn_message.restype = ctypes.c_int
        lib.mlff_painn_message.argtypes = [i32, i32, i32, i64] + [_P] * 13 + [sz, _P]
        lib.mlff_painn_message_backward.restype = ctypes.c_int
        lib.mlff_painn_message_backward.argtypes = [i32, i32, i32, i64] + [_P] * 21 + [sz, _P]
        lib.mlff_painn_update_workspace_size.restype = sz
        lib.mlff_painn_update_workspace_size.argtypes = [i32, i32, i32]
        lib.mlff_painn_update.restype = ctypes.c_int
        lib.mlff_painn_update.argtypes = [i32, i32] + [_P] * 10 + [sz, _P]
        lib.mlff_painn_update_backward.restype = ctypes.c_int
        lib.mlff_painn_update_backward.argtypes = [i32, i32] + [_P] * 17 + [sz, _P]
        lib.mlff_autotune.restype = ctypes.c_int
        lib.mlff_autotune.argtypes = [ctypes.POINTER(Dims), _P, ctypes.POINTER(System), i64, i32,
                                      ctypes.POINTER(Outputs), _P, sz, _P, i32, ctypes.POINTER(i32),
                                      ctypes.POINTER(ctypes.c_double)]
        lib.mlff_autotune_query.restype = ctypes.c_int
        lib.mlff_autotune_query.argtypes = [i32, i32, i32, ctypes.POINTER(i32)]
        lib.mlff_autotune_set.restype = ctypes.c_int
        lib.mlff_autotune_set.argtypes = [i32, i32, i32, i32]
        lib.mlff_autotune_query_shape.restype = ctypes.c_int
        lib.mlff_autotune_query_shape.argtypes = [i32, i32, i32, ctypes.POINTER(i32), ctypes.POINTER(i32)]
        lib.mlff_autotune_set_shape.restype = ctypes.c_int
        lib.mlff_autotune_set_shape.argtypes = [i32, i32, i32, i32, i32]
        lib.mlff_autotune_reset.restype = ctypes.c_int
        lib.mlff_autotune_reset.argtypes = []
        lib.mlff_force_stats_workspace_size.restype = sz
        lib.mlff_force_stats_workspace_size.argtypes = []
        lib.mlff_force_stats.restype = ctypes.c_int
        lib.mlff_force_stats.argtypes = [_P, _P, i64, _P, _P, _P, sz, _P]
        lib.mlff_debug_stall_test.restype = ctypes.c_int
        lib.mlff_debug_stall_test.argtypes = [i32]
        lib.mlff_radius_graph_noalloc.restype = ctypes.c_int
        lib.mlff_radius_graph_noalloc.argtypes = [ctypes.POINTER(System), ctypes.c_float, i64, _P, _P, _P, _P]
        _lib = lib
        return lib


def check(code: int):
    if code != OK:
        msg = load().mlff_last_error_string().decode(errors="replace")
        raise MLFFError(code, msg)


def last_error() -> str:
    return load().mlff_last_error_string().decode(errors="replace")


class Profile:
    """Context manager: per-kind kernel milliseconds and launch counts of
    the library calls made inside it (CUDA events on the launching stream)."""

    def __enter__(self):
        check(load().mlff_profile_begin())
        return self

    def __exit__(self, *exc):
        n = len(PROFILE_KINDS)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int64 * n)()
        check(load().mlff_profile_end(ms, cnt, n))
        self.ms = {k: ms[i] for i, k in enumerate(PROFILE_KINDS)}
        self.launches = {k: int(cnt[i]) for i, k in enumerate(PROFILE_KINDS)}
        return False


def ptr(t) -> Optional[int]:
    return None if t is None else t.data_ptr()
