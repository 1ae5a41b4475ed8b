"""ctypes binding of libsed_gb300.so (the C ABI declared in include/sed_capi.h).

There is no fallback: if the CUDA library is missing or cannot be loaded the
import of any compute entry point raises, so a GPU run can never silently
route around the device kernels.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsed_gb300.so")

SED_OK = 0
SED_ERR_ARG = 1
SED_ERR_CUDA = 2
SED_ERR_NOMEM = 3
SED_ERR_NOT_CONVERGED = 4
SED_ERR_LIMIT = 5
SED_ERR_NOT_HERMITIAN = 6
SED_ERR_TIMEOUT = 7
PREC_FP64 = 0
PREC_MIXED = 1

FIELD_REPS, FIELD_STAB_ORDER, FIELD_STAB_PTR, FIELD_STAB_G, FIELD_STAB_PHASE = 0, 1, 2, 3, 4
FIELD_REP_RANK, FIELD_REP_SYM, FIELD_REP_AMP = 5, 6, 7


class SEDError(RuntimeError):
    """A non-zero status from the C ABI; ``code`` is the SED_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[sed status {code}] {msg}")
        self.code = code


class sed_solve_info(C.Structure):
    _fields_ = [("n_restarts", C.c_int32), ("n_matvec", C.c_int32), ("n_matvec_fp64", C.c_int32),
                ("converged", C.c_int32), ("max_residual", C.c_double), ("max_delta_polish", C.c_double),
                ("seconds", C.c_double)]


# (name, restype, argtypes) of every exported entry point in include/sed_capi.h
_p, _i32, _i64, _u64, _dbl = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double
SIGNATURES = [
    ("sed_last_error", C.c_char_p, []),
    ("sed_api_version", _i32, []),
    ("sed_device_info", _i32, [_p, _p, _p, _p]),
    ("sed_group_create", _i32, [_i32, _i32, _p, _p, _i32, _i32, _p]),
    ("sed_group_inverse", _i32, [_p, _p]),
    ("sed_group_destroy", None, [_p]),
    ("sed_catalog_build", _i32, [_p, _i32, _p]),
    ("sed_catalog_build_species", _i32, [_p, _i32, _i32, _i32, _p]),
    ("sed_catalog_species", _i32, [_p, _p, _p, _p]),
    ("sed_catalog_lookup", _i32, [_p, _i64, _p, _p, _p, _p]),
    ("sed_catalog_info", _i32, [_p, _p, _p, _p]),
    ("sed_catalog_get", _i32, [_p, _i32, _p, _i64]),
    ("sed_catalog_update_phases", _i32, [_p, _p]),
    ("sed_catalog_set_stream", _i32, [_p, _p]),
    ("sed_catalog_destroy", None, [_p]),
    ("sed_sector_build", _i32, [_p, _p, _dbl, _p, _p]),
    ("sed_sector_build_group", _i32, [_p, _p, _p, _dbl, _p, _p]),
    ("sed_sector_get", _i32, [_p, _p, _p, _p]),
    ("sed_sector_project", _i32, [_p, _i64, _p, _p, _p]),
    ("sed_sector_expand_fock", _i32, [_p, _p, _i64, _dbl, _p, _i64, _i32, _p]),
    ("sed_position_operator", _i32, [_p, _p, _p, _p, _p]),
    ("sed_fock_overlaps", _i32, [_p, C.c_int, _p, C.c_int, C.c_int64, C.c_int, _p]),
    ("sed_sector_destroy", None, [_p]),
    ("sed_op_create", _i32, [_p, _i32, _p, _p, _i32, _p, _p, _i32, _p]),
    ("sed_terms_validate", _i32, [_p, _i32, _p, _p]),
    ("sed_op_apply", _i32, [_p, _p, _p, _i64, _i32]),
    ("sed_op_set_apply_shape", _i32, [_p, _i32, _i32]),
    ("sed_op_apply_shape", _i32, [_p, _i32, _p, _p]),
    ("sed_op_info", _i32, [_p, _p, _p, _p]),
    ("sed_op_set_hop_table", _i32, [_p, _i32]),
    ("sed_op_hop_table_info", _i32, [_p, _p, _p, _p]),
    ("sed_op_set_stream", _i32, [_p, _p]),
    ("sed_op_set_priority", _i32, [_p, _i32]),
    ("sed_op_set_sm_limit", _i32, [_p, _i32]),
    ("sed_op_apply_orbit", _i32, [_p, _p, _p]),
    ("sed_op_apply_noalloc", _i32, [_p, _p, _p, _i64]),
    ("sed_op_destroy", None, [_p]),
    ("sed_solve", _i32, [_p, _i32, _dbl, _i32, _i32, _u64, _p, _p, _p]),
    ("sed_batch_create", _i32, [_p, _i32, _p, _i32, _p, _p, _i32, _i32, _i32, _i32, _p]),
    ("sed_batch_run", _i32, [_p, _i32, _p, _p, _p, _p, _dbl, _i32, _p, _p, _p, _p, _p]),
    ("sed_batch_run_vectors", _i32, [_p, _i32, _p, _p, _p, _p, _dbl, _i32, _p, _p, _p, _p, _p, _p, _i64]),
    ("sed_batch_run_device_vectors", _i32, [_p, _i32, _p, _p, _p, _p, _dbl, _i32, _p, _p, _p, _p, _p, _p, _i64]),
    ("sed_batch_last_stats", _i32, [_p, _p, _p, _p]),
    ("sed_batch_last_info", _i32, [_p, _p, _p, _p]),
    ("sed_batch_graph_info", _i32, [_p, _p, _p]),
    ("sed_batch_set_x_in_shared_memory", _i32, [_p, _i32]),
    ("sed_batch_set_hop_table", _i32, [_p, _i32]),
    ("sed_batch_set_site_gauge", _i32, [_p, _i32]),
    ("sed_batch_set_shape", _i32, [_p, _i32, _i32]),
    ("sed_batch_shape", _i32, [_p, _p, _p, _p]),
    ("sed_batch_last_gauge", _i32, [_p, _p]),
    ("sed_batch_run_device", _i32, [_p, _i32, _p, _p, _p, _p, _dbl, _i32, _p, _p, _p, _p, _p]),
    ("sed_batch_set_stream", _i32, [_p, _p]),
    ("sed_batch_info", _i32, [_p, _p, _p, _p]),
    ("sed_batch_destroy", None, [_p]),
    ("sed_batch_ring_start", _i32, [_p, _i32, _i32, _i32]),
    ("sed_batch_ring_submit", _i32, [_p, _p, _p, _p, _u64, _p]),
    ("sed_batch_ring_wait", _i32, [_p, _i64, _i32, _p, _p, _p]),
    ("sed_batch_ring_info", _i32, [_p, _p, _p, _p]),
    ("sed_batch_ring_stop", _i32, [_p]),
    ("sed_server_create", _i32, [_dbl, _i32, _i32, _i64, _i32, _dbl, _p]),
    ("sed_server_add_family", _i32, [_p, _p, _i32, _p, _p, _i32, _p, _p, _i32, _p]),
    ("sed_server_submit", _i32, [_p, _i32, _p, _p, _p, _u64, _i32, _p]),
    ("sed_server_wait", _i32, [_p, _i64, _i32, _p, _p, _p]),
    ("sed_server_next", _i32, [_p, _i32, _p, _p, _p, _p]),
    ("sed_server_stats", _i32, [_p, _p, _p, _p, _p]),
    ("sed_server_destroy", None, [_p]),
]

_lib = None


def load():
    """Load libsed_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                           "(python -m realspace_exactdiagonalization_gb300.build_lib); there is no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        if not hasattr(lib, name):
            continue  # reported by tests/test_abi.py, which requires every declared symbol
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != SED_OK:
        msg = load().sed_last_error()
        raise SEDError(status, msg.decode() if msg else "unknown error")


def ptr(a):
    """ctypes pointer of a numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)
