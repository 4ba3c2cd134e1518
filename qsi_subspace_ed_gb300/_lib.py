"""ctypes binding of libqsi_ed.so (the C-ABI declared in include/qsi_ed.h).

The library is the only compute path: if it is missing the import fails with
an explicit error, and every non-OK status raises QsiError carrying the
library's last-error text.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libqsi_ed.so"

QSI_OK, QSI_INVALID_ARG, QSI_OOM, QSI_CUDA_ERROR, QSI_NOT_CONVERGED, QSI_TIMEOUT, QSI_IO_ERROR, QSI_NOT_FOUND = range(8)
STATUS_NAMES = ["OK", "INVALID_ARG", "OOM", "CUDA_ERROR", "NOT_CONVERGED", "TIMEOUT", "IO_ERROR", "NOT_FOUND"]
QSI_PTR_HOST, QSI_PTR_DEVICE = 0, 1
QSI_F64, QSI_F32 = 0, 1
QSI_TUNE_INDEX, QSI_TUNE_LOOKUP = 1, 2
CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


class QsiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"QSI_{name}: {msg}")


class Term(C.Structure):
    """qsi_term: coefficient plus the masks of SymbolicPMROperator."""

    _fields_ = [
        ("c", C.c_double),
        ("x", C.c_uint64 * 2),
        ("z", C.c_uint64 * 2),
        ("up", C.c_uint64 * 2),
        ("down", C.c_uint64 * 2),
        ("sign", C.c_int32),
        ("reserved", C.c_int32),
    ]


class LanczosCfg(C.Structure):
    _fields_ = [
        ("nev", C.c_int32),
        ("ncv", C.c_int32),
        ("max_iter", C.c_int32),
        ("precision", C.c_int32),
        ("tol", C.c_double),
        ("seed", C.c_uint64),
        ("polish_steps", C.c_int32),
        ("want_vectors", C.c_int32),
        ("block", C.c_int32),
        ("reserved", C.c_int32),
    ]


class Report(C.Structure):
    _fields_ = [
        ("converged", C.c_int32),
        ("restarts", C.c_int32),
        ("applies", C.c_int64),
        ("residual", C.c_double * 64),
        ("seconds", C.c_double),
    ]


class Eigval0Cfg(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int32),
        ("min_iterations", C.c_int32),
        ("abs_tol", C.c_double),
        ("rel_tol", C.c_double),
        ("seed", C.c_uint64),
        ("calc_eigenvector", C.c_int32),
        ("reserved", C.c_int32),
    ]


_P = C.c_void_p
_I32, _I64, _U64, _D = C.c_int32, C.c_int64, C.c_uint64, C.c_double

# name -> argtypes (restype is qsi_status = int unless listed in _RESTYPES)
SIGNATURES = {
    "qsi_version": [],
    "qsi_last_error": [C.c_char_p, C.c_size_t],
    "qsi_term_compile": [C.c_char_p, _P, _I32, _D, C.POINTER(Term)],
    "qsi_term_parse": [C.c_char_p, _D, C.POINTER(Term)],
    "qsi_term_mul": [C.POINTER(Term), C.POINTER(Term)],
    "qsi_term_apply_state": [C.POINTER(Term), _P, C.POINTER(_I32)],
    "qsi_h5_read_basis": [C.c_char_p, C.c_char_p, _P, _I64, C.POINTER(_I64)],
    "qsi_h5_read_f64": [C.c_char_p, C.c_char_p, _P, _I64, C.POINTER(_I64), _P, C.POINTER(_I32)],
    "qsi_h5_write_basis": [C.c_char_p, C.c_char_p, _P, _I64, _I32],
    "qsi_h5_write_eigs": [C.c_char_p, _P, _I64, _P, _I64, _I64, C.c_char_p, C.c_char_p],
    "qsi_h5_write_f64": [C.c_char_p, C.c_char_p, _P, _P, _I32, _I32],
    "qsi_h5_write_string": [C.c_char_p, C.c_char_p, C.c_char_p, _I32],
    "qsi_h5_read_string": [C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t],
    "qsi_csv_read_basis": [C.c_char_p, _P, _I64, C.POINTER(_I64)],
    "qsi_enumerate_basis": [_I32, _P, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32,
                            C.POINTER(C.POINTER(C.c_uint64)), C.POINTER(_I64)],
    "qsi_free_host": [_P],
    "qsi_enumerate_basis_gpu": [_I32, _P, _I32, _I32, _P, _I32, _P, _I32, C.POINTER(C.POINTER(C.c_uint64)),
                                C.POINTER(_I64)],
    "qsi_partition_basis": [_P, _I64, _P, _I32, _P, _P, _P, _I32, C.POINTER(_I32)],
    "qsi_partition_basis_h5": [C.c_char_p, C.c_char_p, C.c_char_p, _P, _I32],
    "qsi_basis_create": [_P, _I64, _I32, C.POINTER(_P)],
    "qsi_basis_destroy": [_P],
    "qsi_basis_dim": [_P, C.POINTER(_I64)],
    "qsi_basis_search": [_P, _P, _I64, _P, _I32, _P],
    "qsi_basis_index": [_P, _I32, _I32],
    "qsi_basis_info": [_P, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I64)],
    "qsi_op_create": [_P, _P, _I32, C.POINTER(_P)],
    "qsi_op_destroy": [_P],
    "qsi_family_create": [_P, _P, _I32, _P, _I32, _I32, C.POINTER(_P)],
    "qsi_family_destroy": [_P],
    "qsi_family_member": [_P, _P, C.POINTER(_P)],
    "qsi_family_stats": [_P, C.POINTER(_I64), C.POINTER(_I64)],
    "qsi_family_set_min_rows": [_P, _I64],
    "qsi_op_materialise": [_P, _I32, C.POINTER(_I64)],
    "qsi_op_apply": [_P, _P, _P, _I32, _I32, _P],
    "qsi_op_apply_static": [_P, _P, _P, _I32],
    "qsi_op_apply_batched": [_P, _P, _P, _I32, _I32, _I32, _I32, _P],
    "qsi_op_set_kernel": [_P, _I32, _I32, _I32],
    "qsi_op_info": [_P, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32)],
    "qsi_op_write_mtx": [_P, C.c_char_p, _D, C.POINTER(_I64)],
    "qsi_expectations": [_P, _P, _P, _I32, _P, _I32, _P, _P],
    "qsi_op_set_tuning": [_P, _I32, _I32, _I32, _I32],
    "qsi_op_get_tuning": [_P, _I32, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32),
                          C.POINTER(_I32), C.POINTER(_I32)],
    "qsi_op_autotune": [_P, _P, _P, _I32, _I32, _I32, _I32, C.c_char_p, C.c_size_t],
    "qsi_op_triplets": [_P, _D, _P, _P, _P, _I64, C.POINTER(_I64)],
    "qsi_op_count_misses": [_P, C.POINTER(_I64)],
    "qsi_op_connectivity": [_P, C.POINTER(_I64), C.POINTER(_I64)],
    "qsi_lanczos_solve": [_P, C.POINTER(LanczosCfg), _P, _P, C.POINTER(Report)],
    "qsi_eigval0": [_P, C.POINTER(Eigval0Cfg), C.POINTER(_D), _P, C.POINTER(_I32)],
    "qsi_eigval0_checkpointed": [_P, C.POINTER(Eigval0Cfg), C.c_char_p, _I32, _I32, _D, C.POINTER(_D), _P,
                                 C.POINTER(_I32)],
    "qsi_ftlm_run": [_P, _I32, _P, _I32, _U64, _I32, _P, _P],
    "qsi_ftlm_run_blocks": [_P, _I32, _P, _I32, _U64, _I32, _I32, _P, _P],
    "qsi_tridiag_ritz": [_P, _P, _I32, _I32, _P, _P],
}
_RESTYPES = {"qsi_version": C.c_char_p, "qsi_free_host": None}

_lib = None


def load() -> C.CDLL:
    """Loads libqsi_ed.so from the package directory (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it first (python -m qsi_subspace_ed_gb300._build, "
            "or __graft_entry__.build()); there is no fallback compute path")
    lib = C.CDLL(str(LIB_PATH))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    load().qsi_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != QSI_OK:
        raise QsiError(status, last_error())


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def ptr(a) -> C.c_void_p:
    """Address of a numpy array or torch tensor (contiguous)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def exported_symbols():
    return list(SIGNATURES)


if os.environ.get("QSI_EAGER_LOAD"):
    load()
