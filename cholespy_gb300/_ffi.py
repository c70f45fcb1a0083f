"""ctypes binding of the gbchol C ABI (include/gbchol.h).

The shared library is built in-tree by ``cholespy_gb300._build`` (or
``__graft_entry__.build()``). There is no fallback: if the library is missing
every entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB = None
LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgbchol.so"

OK, EINVAL, ENOTPOSDEF, ECUDA, ENOMEM, ETIMEOUT, ESTATE, EINTERNAL = range(8)
STORE_F32, STORE_F64, STORE_A64 = 1, 2, 4
MAX_RHS = 128


class Info(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("device", C.c_int32),
        ("nnz_a", C.c_int64),
        ("nnz_l", C.c_int64),
        ("levels_lower", C.c_int32),
        ("levels_upper", C.c_int32),
        ("n_supernodes", C.c_int32),
        ("max_supernode", C.c_int32),
        ("factor_flops", C.c_double),
        ("factor_seconds", C.c_double),
        ("analysis_seconds", C.c_double),
        ("store", C.c_int32),
        ("top_rows", C.c_int32),
        ("top_units", C.c_int32),
        ("top_blocks", C.c_int64),
        ("launches_per_solve", C.c_int32),
    ]


class BatchOptions(C.Structure):
    """gbchol_batch_options: the row sweeps' group budget, wavefront skew and lane-mode variant."""
    _fields_ = [
        ("group_bytes", C.c_int64),
        ("skew", C.c_int32),
        ("row_variant", C.c_int32),
    ]


class RefineStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("converged", C.c_int32),
        ("max_rel_residual", C.c_double),
    ]


def _declare(lib):
    P, I32, I64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "gbchol_last_error": (C.c_char_p, []),
        "gbchol_version": (C.c_char_p, []),
        "gbchol_create": (C.c_int, [I32, I64, P, P, P, I32, I32, C.POINTER(P)]),
        "gbchol_create_device": (C.c_int, [I32, I64, P, P, P, I32, I32, C.POINTER(P)]),
        "gbchol_create_from_factor": (C.c_int, [I32, P, P, P, P, I32, C.POINTER(P)]),
        "gbchol_destroy": (C.c_int, [P]),
        "gbchol_solve": (C.c_int, [P, I32, I32, P, P, P]),
        "gbchol_solve_refined": (C.c_int, [P, I32, P, P, D, I32, P, C.POINTER(RefineStats)]),
        "gbchol_get_info": (C.c_int, [P, C.POINTER(Info)]),
        "gbchol_get_levels": (C.c_int, [P, I32, P, P, P]),
        "gbchol_get_factor": (C.c_int, [P, P, P, P, P]),
        "gbchol_check": (C.c_int, [P]),
        "gbchol_reserve": (C.c_int, [P, I32]),
        "gbchol_replan": (C.c_int, [P, I32, I32, I32]),
        "gbchol_refactorize": (C.c_int, [P, I64, P, P, P, I32]),
        "gbchol_factor_refactorize": (C.c_int, [P, I64, P, P, P, I32, I32]),
        "gbchol_autotune": (C.c_int, [P, I32, I32, P, I32, I32, C.POINTER(I32)]),
        "gbchol_autotune_sweeps": (C.c_int, [P, I32, I32, I32, C.POINTER(I32)]),
        "gbchol_factorize": (C.c_int, [I32, I64, P, P, P, I32, I32, C.POINTER(P)]),
        "gbchol_factor_info": (C.c_int, [P, C.POINTER(I32), C.POINTER(I64), C.POINTER(I32),
                                         C.POINTER(D)]),
        "gbchol_factor_export": (C.c_int, [P, P, P, P, P]),
        "gbchol_factor_free": (C.c_int, [P]),
        "gbchol_factor_solve": (C.c_int, [P, I32, I32, P, P, I32]),
        "gbchol_batch_create": (C.c_int, [I32, P, P, I32, C.POINTER(P)]),
        "gbchol_batch_create_ex": (C.c_int, [I32, P, P, I32, C.POINTER(BatchOptions), C.POINTER(P)]),
        "gbchol_batch_set_io": (C.c_int, [P, P, P]),
        "gbchol_batch_solve": (C.c_int, [P, P]),
        "gbchol_batch_info": (C.c_int, [P, C.POINTER(I32), C.POINTER(I64), C.POINTER(I64)]),
        "gbchol_batch_check": (C.c_int, [P, P]),
        "gbchol_batch_destroy": (C.c_int, [P]),
        "gbchol_grad_values": (C.c_int, [I32, I64, I32, P, P, P, P, P, I32, I32, P]),
        "gbchol_selftest_wait": (C.c_int, [I32, C.POINTER(I32)]),
        "gbchol_solve_noalloc": (C.c_int, [P, I32, I32, P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib():
    """The loaded libgbchol (raises ImportError when it has not been built)."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m cholespy_gb300._build` "
                "(or __graft_entry__.build()); there is no non-CUDA fallback.")
        handle = C.CDLL(str(LIB_PATH))
        _declare(handle)
        _LIB = handle
    return _LIB


def last_error() -> str:
    msg = lib().gbchol_last_error()
    return msg.decode() if msg else ""


def check(status: int) -> None:
    """Raise the Python exception matching a gbchol status."""
    if status == OK:
        return
    msg = last_error() or f"gbchol error {status}"
    if status in (EINVAL, ENOTPOSDEF):
        raise ValueError(msg)
    if status == ENOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg)
