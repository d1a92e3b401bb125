"""ctypes binding of libkapdqmc_gpu.so (the C ABI in include/kapdqmc.h).

There is no CPU fallback: if the library is missing or no GPU is usable the
calls raise.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libkapdqmc_gpu.so"

KDQ_OK, KDQ_ERR_ARG, KDQ_ERR_CUDA, KDQ_ERR_NUMERIC, KDQ_ERR_STATE, KDQ_ERR_NOGPU = range(6)

# Every function the header declares, with its ctypes signature.
_SIGS = {
    "kdq_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_int32, C.c_int32]),
    "kdq_destroy": (None, [C.c_void_p]),
    "kdq_last_error": (C.c_char_p, [C.c_void_p]),
    "kdq_set_fields": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_get_fields": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_set_rng": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64]),
    "kdq_set_tape": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_phy_update": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t]),
    "kdq_init": (C.c_int, [C.c_void_p]),
    "kdq_sweep": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "kdq_get_obs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_synchronize": (C.c_int, [C.c_void_p]),
    "kdq_n_obs": (C.c_int, [C.c_void_p]),
    "kdq_get_green": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    "kdq_get_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "kdq_enable_accept_log": (C.c_int, [C.c_void_p, C.c_size_t]),
    "kdq_get_accept_log": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_get_drift": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_get_log_det": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "kdq_slmc_enable": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "kdq_get_slmc_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "kdq_scee_enable": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double,
                                  C.c_int32]),
    "kdq_scee_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    "kdq_scee_get_green": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t]),
    "kdq_dop_enable": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                 C.c_double, C.c_int32]),
    "kdq_dop_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    "kdq_set_measure_full": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_cnn_forward": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
    "kdq_cnn_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                               C.c_int32]),
    "kdq_cnn_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                C.c_float, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int32]),
    "kdq_stream": (C.c_void_p, [C.c_void_p]),
    "kdq_set_graphs": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_set_sweep_launch": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_set_tiles": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_get_tiles": (C.c_int, [C.c_void_p]),
    "kdq_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "kdq_group_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_int32]),
    "kdq_group_sweep": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "kdq_group_synchronize": (C.c_int, [C.c_void_p]),
    "kdq_group_last_error": (C.c_char_p, [C.c_void_p]),
    "kdq_group_destroy": (None, [C.c_void_p]),
    "kdq_set_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_enable_phase_timing": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_get_phase_cycles": (C.c_int, [C.c_void_p, C.c_void_p]),
    "kdq_grover_det": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                 C.c_void_p, C.c_int32]),
    "kdq_grover_det_chains": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "kdq_keep_middle_green": (C.c_int, [C.c_void_p, C.c_int32]),
    "kdq_grover_det_middle": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "kdq_grover_det_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                         C.c_int32, C.c_void_p, C.c_void_p]),
}


class ModelDesc(C.Structure):
    """kdq_model_desc."""
    _fields_ = [
        ("kind", C.c_int32), ("lattice", C.c_int32), ("site", C.c_int32 * 2),
        ("Ns", C.c_int32), ("Nt", C.c_int32), ("z", C.c_int32),
        ("g_complex", C.c_int32), ("k_complex", C.c_int32), ("n_nodes", C.c_int32),
        ("nodes", C.c_void_p), ("alpha", C.c_void_p), ("gamma", C.c_void_p), ("eta", C.c_void_p),
        ("a", C.c_double), ("Ht", C.c_double), ("U", C.c_double), ("V", C.c_double),
        ("eK", C.c_void_p), ("eKinv", C.c_void_p), ("HalfeK", C.c_void_p),
        ("HalfeKinv", C.c_void_p), ("K", C.c_void_p), ("Pt", C.c_void_p), ("bonds", C.c_void_p),
    ]


class Stats(C.Structure):
    """kdq_stats."""
    _fields_ = [("proposals", C.c_int64), ("accepted", C.c_int64), ("recomputes", C.c_int64),
                ("max_drift", C.c_double), ("seconds", C.c_double)]


_lib = None


def load():
    """Load the library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        from .build import build
        build()
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class KdqError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"kapdqmc error {code}: {msg}")
        self.code = code


def check(rc, handle=None):
    if rc != KDQ_OK:
        msg = load().kdq_last_error(handle)
        raise KdqError(rc, msg.decode() if msg else "")
