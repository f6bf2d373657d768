"""ctypes binding of libqmbx.so (declared in include/qmbx.h).

The library must have been built (``__graft_entry__.build()`` or
``python qmb-public_gb300/_build.py``); loading fails loudly otherwise.  There
is no CPU fallback: every device entry point runs the CUDA kernels.
"""

from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqmbx.so")

QMBX_OK = 0
QMBX_ERR_ARGUMENT = 1
QMBX_ERR_CUDA = 2
QMBX_ERR_WORKSPACE = 3
QMBX_ERR_DEVICE = 4

_lib: ctypes.CDLL | None = None

# name -> (restype, argtypes)
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_U64 = ctypes.c_uint64
_PU64 = ctypes.POINTER(ctypes.c_uint64)
_PI64 = ctypes.POINTER(ctypes.c_int64)

SIGNATURES: dict[str, tuple] = {
    "qmbx_version": (ctypes.c_int, []),
    "qmbx_last_error": (ctypes.c_char_p, []),
    "qmbx_table_bytes": (ctypes.c_int, [_P, _P, _I64, _I32, _I32, _PU64]),
    "qmbx_table_build": (ctypes.c_int, [_P, _P, _P, _I64, _I32, _I32, _P, _U64]),
    "qmbx_table_counts": (ctypes.c_int, [_P, _PI64]),
    "qmbx_table_check": (ctypes.c_int, [_P, _U64]),
    "qmbx_table_hermitian": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
    "qmbx_apply_within_workspace": (ctypes.c_int, [_P, _I64, _I64, _PU64]),
    "qmbx_apply_within": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P, _I64, _I32, _P, _P, _U64, _P]),
    "qmbx_apply_within_static": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P, _I64, _I32, _P, _P]),
    "qmbx_apply_within_adjoint": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _I64, _I32, _P, _P, _U64, _P]),
    "qmbx_apply_within_f32c": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P, _I64, _I32, _I32, _P, _P, _P, _U64, _P]),
    "qmbx_apply_within_adjoint_f32c": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _I64, _I32, _I32, _P, _P, _P, _U64, _P]),
    "qmbx_diagonal_term": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P]),
    "qmbx_hitlog_bytes": (ctypes.c_int, [_P, _I64, _I64, _I32, _I64, _PU64]),
    "qmbx_hitlog_count": (ctypes.c_int, [_P, _P, _P]),
    "qmbx_apply_within_logged": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P, _I64, _I32, _P, _P, _U64, _I64, _P]),
    "qmbx_apply_within_f32c_logged": (ctypes.c_int, [_P, _P, _P, _P, _I64, _P, _I64, _I32, _I32, _P, _P, _P, _U64,
                                                     _I64, _P]),
    "qmbx_apply_within_adjoint_logged": (ctypes.c_int, [_P, _P, _P, _U64, _I64, _I64, _I64, _I32, _P, _P, _P]),
    "qmbx_apply_within_adjoint_f32c_logged": (ctypes.c_int, [_P, _P, _P, _U64, _I64, _I64, _I64, _I32, _I32, _P, _P,
                                                             _P, _P]),
    "qmbx_matrix_workspace": (ctypes.c_int, [_P, _I64, _PU64]),
    "qmbx_matrix_count": (ctypes.c_int, [_P, _P, _P, _I64, _P, _PI64, _P, _U64, _P]),
    "qmbx_matrix_fill": (ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _P, _P, _U64, _P]),
    "qmbx_matrix_apply": (ctypes.c_int, [_I64, _P, _P, _P, _P, _P, _P]),
    "qmbx_matrix_apply_many": (ctypes.c_int, [_I64, _I64, _I32, _P, _P, _P, _P, _P, _P]),
    "qmbx_find_relative_workspace": (ctypes.c_int, [_P, _I64, _I64, _I64, _PU64]),
    "qmbx_find_relative": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _P, _I64, _P, _PI64, _P, _U64, _PU64, _P]),
    "qmbx_find_relative_stats": (ctypes.c_int, [_PI64]),
    "qmbx_pt2_workspace": (ctypes.c_int, [_P, _I64, _I64, _PU64]),
    "qmbx_pt2": (ctypes.c_int, [_P, _P, _P, _P, _I64, _I64, _P, _PI64, _P, _U64, _PU64, _P]),
    "qmbx_single_relative_workspace": (ctypes.c_int, [_P, _I64, _PU64]),
    "qmbx_single_relative": (ctypes.c_int, [_P, _P, _P, _I64, _U64, _P, _P, _U64, _P]),
    "qmbx_sampler_log_amplitude": (ctypes.c_int, [_I64, _I32, _I32, _I32, _P, _P, _P, _P]),
    "qmbx_sampler_log_amplitude_grad": (ctypes.c_int, [_I64, _I32, _I32, _I32, _P, _P, _P, _P, _P]),
    "qmbx_sampler_site": (ctypes.c_int, [_I64, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                         _P]),
    "qmbx_sampler_take": (ctypes.c_int, [_I64, _I64, _I32, _I32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                         _P, _I64, _P]),
    "qmbx_profile_enable": (ctypes.c_int, [_I32]),
    "qmbx_profile_read": (ctypes.c_int, [_PI64, _PI64, ctypes.POINTER(ctypes.c_double)]),
}

PROFILE_GROUPS = ("enumerate", "keys", "select", "other", "diagonal", "sort", "spmv")


def profile_enable(on: bool) -> None:
    """Start (and reset) or stop per-group kernel timing with CUDA events."""
    check(library().qmbx_profile_enable(1 if on else 0))


def profile_read() -> dict:
    """Launch counter and per-group (count, milliseconds) since the last profile_enable."""
    launches = ctypes.c_int64()
    counts = (ctypes.c_int64 * len(PROFILE_GROUPS))()
    ms = (ctypes.c_double * len(PROFILE_GROUPS))()
    check(library().qmbx_profile_read(ctypes.byref(launches), counts, ms))
    return {"launches": launches.value,
            "groups": {g: (counts[k], ms[k]) for k, g in enumerate(PROFILE_GROUPS)}}


FIND_STATS = ("records", "walks", "sort_passes", "sort_bytes", "selected", "rows_out")


def find_relative_stats() -> dict:
    """Figures of this thread's last find_relative call (see qmbx_find_relative_stats)."""
    vals = (ctypes.c_int64 * len(FIND_STATS))()
    check(library().qmbx_find_relative_stats(vals))
    return dict(zip(FIND_STATS, list(vals)))


class QmbxError(RuntimeError):
    """An entry point of libqmbx.so returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def library() -> ctypes.CDLL:
    """Load libqmbx.so (once) and declare its entry points."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status: int) -> None:
    if status != QMBX_OK:
        msg = library().qmbx_last_error().decode(errors="replace")
        if status == QMBX_ERR_ARGUMENT:
            raise QmbxError(status, msg)
        raise QmbxError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(library(), name)(*args))
