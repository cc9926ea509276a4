"""ctypes binding of ``libepet_gb300.so`` (the C ABI in include/epet_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded,
``lib()`` raises ``RuntimeError`` -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libepet_gb300.so")

EPET_OK = 0
STATUS_NAMES = {0: "EPET_OK", 1: "EPET_ERR_INVALID", 2: "EPET_ERR_CAPACITY", 3: "EPET_ERR_CUDA",
                4: "EPET_ERR_UNSUPPORTED", 5: "EPET_ERR_TIMEOUT", 6: "EPET_ERR_OVERFLOW"}


class EpetError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Setup(C.Structure):
    _fields_ = [("pos0x", C.c_float), ("pos1x", C.c_float), ("na", C.c_int32),
                ("n0z", C.c_int32), ("n0y", C.c_int32), ("n1z", C.c_int32),
                ("n1y", C.c_int32), ("da", C.c_float), ("segx", C.c_float),
                ("segy", C.c_float), ("segz", C.c_float)]


class Grid(C.Structure):
    _fields_ = [("o", C.c_float * 3), ("d", C.c_float * 3), ("n", C.c_int32 * 3)]


class ProblemC(C.Structure):
    _fields_ = [("setup", Setup), ("grid", Grid), ("nrays", C.c_int32),
                ("ray_mode", C.c_int32), ("seed", C.c_uint64)]


class CsrC(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p)]


class CscC(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("nnz", C.c_int64),
                ("col_ptr", C.c_void_p), ("row", C.c_void_p), ("val", C.c_void_p)]


class Csr16C(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("nnz", C.c_int64),
                ("row_ptr", C.c_void_p), ("base", C.c_void_p), ("scale", C.c_void_p),
                ("delta", C.c_void_p), ("q", C.c_void_p), ("format", C.c_int32)]


class MlemOptions(C.Structure):
    _fields_ = [("max_row_nnz", C.c_int32), ("use_graph", C.c_int32),
                ("value_format", C.c_int32), ("autotune", C.c_int32),
                ("matrix_free", C.c_int32), ("layout", C.c_int32)]


P, VP, I64, I32, F, D, SZ = (C.POINTER(ProblemC), C.c_void_p, C.c_int64, C.c_int32, C.c_float,
                             C.c_double, C.c_size_t)

# name -> argtypes (all return epet_status unless listed in _RESTYPES)
SIGNATURES = {
    "epet_last_error": [],
    "epet_version": [],
    "epet_launch_count": [],
    "epet_device_allocations": [],
    "epet_debug_fail_allocations": [C.c_longlong],
    "epet_problem_validate": [P],
    "epet_trig_table": [P, VP, VP],
    "epet_dump_uniforms": [P, VP, I64, VP, VP],
    "epet_rays": [P, VP, I64, VP, VP],
    "epet_workqueue_count": [P, VP, I64, VP, C.POINTER(C.c_int64), VP],
    "epet_workqueue_fill": [P, VP, I64, VP, VP, VP, VP],
    "epet_sm_values": [P, VP, I64, VP, VP, VP, VP, SZ, VP],
    "epet_sm_values_workspace_size": [P, I64],
    "epet_sm_build": [P, VP, I64, C.POINTER(CsrC), I64, C.POINTER(C.c_int64), I32, VP, SZ, VP],
    "epet_sm_build_workspace_size": [P, I64, I32],
    "epet_project_forward": [P, VP, I64, VP, VP, I32, VP, SZ, VP],
    "epet_project_back": [P, VP, I64, VP, VP, I32, VP, SZ, VP],
    "epet_project_mlem": [P, VP, I64, VP, VP, VP, VP, I32, VP, SZ, VP],
    "epet_sensitivity": [P, VP, I64, VP, VP, I32, VP, SZ, VP],
    "epet_coo_sort": [VP, VP, VP, I64, VP, SZ, VP],
    "epet_coo_sort_workspace_size": [I64],
    "epet_coo_sort_noalloc": [VP, VP, VP, I64, VP],
    "epet_coo2csr": [VP, I64, I64, VP, VP],
    "epet_csr2ecsr": [VP, VP, I64, VP, I64, VP],
    "epet_csr_to_csc": [C.POINTER(CsrC), C.POINTER(CscC), VP, SZ, VP],
    "epet_csr_to_csc_workspace_size": [I64, I64, I64],
    "epet_csr16_count": [C.POINTER(CsrC), VP, C.POINTER(C.c_int64), VP],
    "epet_csr_compress": [C.POINTER(CsrC), I32, C.POINTER(Csr16C), VP],
    "epet_csr16_mv": [C.POINTER(Csr16C), F, VP, F, VP, VP],
    "epet_csrmv": [C.c_int, C.POINTER(CsrC), C.POINTER(CscC), F, VP, F, VP, VP],
    "epet_divides": [VP, VP, VP, I64, VP],
    "epet_divides_multiplies": [VP, VP, VP, VP, I64, VP],
    "epet_scales": [VP, F, I64, VP],
    "epet_sum_f64": [VP, I64, VP, VP],
    "epet_coo2csr_i32": [VP, I64, I64, VP, VP],
    "epet_csr2ecsr_i32": [VP, VP, I64, VP, I64, VP],
    "epet_csrmv_i32": [C.c_int, I64, I64, I64, F, VP, VP, VP, VP, F, VP, VP],
    "epet_index_i64_to_i32": [VP, I64, VP, VP],
    "epet_index_i32_to_i64": [VP, I64, VP, VP],
    "epet_csr_expand_rows": [VP, I64, VP, VP, VP],
    "epet_set_constant_geometry": [C.POINTER(Setup), C.POINTER(Grid), I32],
    "epet_get_constant_geometry": [P],
    "epet_mlem_create": [P, VP, VP, I64, VP, C.POINTER(MlemOptions), C.POINTER(VP), VP],
    "epet_mlem_destroy": [VP],
    "epet_mlem_iterate": [VP, I32, C.POINTER(C.c_double), VP],
    "epet_mlem_image": [VP],
    "epet_mlem_get_image": [VP, VP, VP],
    "epet_mlem_set_image": [VP, VP, VP],
    "epet_mlem_stats": [VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
    "epet_mlem_plan": [VP, C.POINTER(C.c_int32)],
    "epet_mlem_layout": [VP, C.POINTER(C.c_int32)],
    "epet_mlem_correction": [VP, VP, VP],
    "epet_mlem_update": [VP, VP, VP],
    "epet_mlem_loglik": [VP, C.POINTER(C.c_double), VP],
    "epet_trim_memory": [C.c_size_t],
    "epet_selftest_division": [I64, C.c_uint64, C.POINTER(C.c_int64), VP],
    "epet_build_counters": [C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
    "epet_ray_steps": [P, VP, I64, VP, C.POINTER(C.c_int64), VP],
    "epet_mlem_batch_create": [I32, VP, VP, VP, VP, VP, C.POINTER(MlemOptions), C.POINTER(VP),
                               VP],
    "epet_mlem_batch_destroy": [VP],
    "epet_mlem_batch_iterate": [VP, I32, VP, VP],
    "epet_mlem_batch_get_image": [VP, I32, VP, VP],
    "epet_mlem_batch_member": [VP, I32],
    "epet_mlem_batch_stats": [VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64), VP],
    "epet_h5_dataset_shape": [C.c_char_p, C.c_char_p, C.POINTER(C.c_int32),
                              C.POINTER(C.c_int64)],
    "epet_h5_read_f32": [C.c_char_p, C.c_char_p, VP, I64],
    "epet_h5_read_measurement": [C.c_char_p, VP, VP, I64, C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64)],
    "epet_h5_write_measurement": [C.c_char_p, VP, I64],
    "epet_h5_write_density": [C.c_char_p, VP, C.POINTER(Grid)],
    "epet_h5_read_density": [C.c_char_p, VP, I64, C.POINTER(Grid)],
    "epet_h5_write_checkpoint": [C.c_char_p, VP, C.POINTER(Grid), I64],
    "epet_h5_read_attribute": [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_double)],
}
_RESTYPES = {
    "epet_last_error": C.c_char_p,
    "epet_version": C.c_char_p,
    "epet_launch_count": C.c_longlong,
    "epet_device_allocations": C.c_longlong,
    "epet_sm_values_workspace_size": SZ,
    "epet_sm_build_workspace_size": SZ,
    "epet_coo_sort_workspace_size": SZ,
    "epet_csr_to_csc_workspace_size": SZ,
    "epet_mlem_image": VP,
    "epet_mlem_batch_member": VP,
}

_LIB = None


def lib() -> C.CDLL:
    """The loaded library.  Raises if it is not built (no fallback)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m epetreco_gb300.build` "
                "(the CUDA library is the only compute path)")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPES.get(name, C.c_int)
        _LIB = L
    return _LIB


def check(status: int) -> None:
    if status != EPET_OK:
        raise EpetError(status, lib().epet_last_error().decode())


def problem_struct(p) -> ProblemC:
    s, g = p.setup, p.grid
    return ProblemC(Setup(s.pos0x, s.pos1x, s.na, s.n0z, s.n0y, s.n1z, s.n1y, s.da, s.segx,
                          s.segy, s.segz),
                    Grid((C.c_float * 3)(*g.origin), (C.c_float * 3)(*g.pitch),
                         (C.c_int32 * 3)(*g.n)),
                    int(p.nrays), int(p.ray_mode), int(p.seed))
