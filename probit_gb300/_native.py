"""ctypes binding of ``libprobit_gb300.so`` (the C-ABI of include/probit_gb300.h
and its DLPack entry points, include/probit_gb300_dlpack.h).

The library is the only compute path: if it is missing or cannot be loaded,
every entry point raises ``NativeLibraryError``; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libprobit_gb300.so"
HEADER = _PKG.parent / "include" / "probit_gb300.h"

PGB_OK = 0
PGB_EINVAL = -1
PGB_ENOMEM = -2
PGB_ECUDA = -3
PGB_ENOTPD = -4
PGB_ENAN = -5
PGB_ETIMEOUT = -6
PGB_EUNSUPPORTED = -7
PGB_ESTATE = -8

KERNEL_EQ = 0
KERNEL_MATERN12 = 1
KERNEL_EQ_PERIODIC = 2

LIK_GAUSSIAN = 0
LIK_PROBIT = 1
LIK_PROBIT_STABLE = 2

MAX_D = 16


class NativeLibraryError(RuntimeError):
    """The CUDA library is missing or failed to load."""


class PgbError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__(f"{where}: {strerror(code)} ({code})")


class Desc(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("d", C.c_int32),
        ("kernel", C.c_int32),
        ("n_lengthscales", C.c_int32),
        ("period", C.c_float),
        ("likelihood", C.c_int32),
        ("j", C.c_int32),
        ("tolerance", C.c_float),
        ("maxiter", C.c_int32),
        ("flags", C.c_int32),
    ]


class Status(C.Structure):
    _fields_ = [
        ("code", C.c_int32),
        ("iterations", C.c_int32),
        ("notpd_col", C.c_int32),
        ("converged", C.c_int32),
    ]


class DLTensor(C.Structure):
    """DLPack's DLTensor (the ``pgb_dltensor`` of include/probit_gb300_dlpack.h)."""

    _fields_ = [
        ("data", C.c_void_p),
        ("device_type", C.c_int32),
        ("device_id", C.c_int32),
        ("ndim", C.c_int32),
        ("dtype_code", C.c_uint8),
        ("dtype_bits", C.c_uint8),
        ("dtype_lanes", C.c_uint16),
        ("shape", C.POINTER(C.c_int64)),
        ("strides", C.POINTER(C.c_int64)),
        ("byte_offset", C.c_uint64),
    ]


_capsule_ptr = C.pythonapi.PyCapsule_GetPointer
_capsule_ptr.restype = C.c_void_p
_capsule_ptr.argtypes = [C.py_object, C.c_char_p]


def dlpack_tensor(obj):
    """(capsule, address of its DLTensor) for a torch tensor or any object
    with ``__dlpack__`` (legacy, unversioned capsule).  The capsule must stay
    referenced while the address is used; the producer keeps ownership."""
    if hasattr(obj, "__dlpack__"):
        cap = obj.__dlpack__()
    else:
        cap = obj
    return cap, _capsule_ptr(cap, b"dltensor")


_VP = C.c_void_p
_SIGS = {
    "pgb_version": (C.c_char_p, []),
    "pgb_strerror": (C.c_char_p, [C.c_int]),
    "pgb_theta_size": (C.c_int, [C.POINTER(Desc)]),
    "pgb_gp_create": (C.c_int, [C.POINTER(Desc), C.POINTER(_VP)]),
    "pgb_gp_destroy": (C.c_int, [_VP]),
    "pgb_gp_status": (C.c_int, [_VP, C.POINTER(Status), _VP]),
    "pgb_gp_set_max_blocks": (C.c_int, [_VP, C.c_int32]),
    "pgb_gram": (C.c_int, [C.POINTER(Desc), _VP, _VP, C.c_int32, _VP, C.c_int32, _VP, C.c_int64, _VP]),
    "pgb_gram_noalloc": (C.c_int, [C.POINTER(Desc), _VP, _VP, C.c_int32, _VP, C.c_int32, _VP, C.c_int64, _VP]),
    "pgb_log_likelihood": (C.c_int, [C.POINTER(Desc), _VP, _VP, _VP, C.c_int32, _VP, _VP, _VP, _VP, _VP]),
    "pgb_weight": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_precision": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_approximate_posterior": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_objective": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_vb_weight": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_vb_objective": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_vb_value_and_grad": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_value_and_grad": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_factor": (C.c_int, [_VP, _VP]),
    "pgb_predict": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, C.c_int32, _VP, _VP, C.c_int32, _VP]),
    "pgb_predict_distributions": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, C.c_int32, _VP, _VP, _VP, C.c_int32,
                                             _VP]),
    "pgb_predictive_distributions": (C.c_int, [C.POINTER(Desc), _VP, _VP, _VP, C.c_int32, _VP, _VP]),
    "pgb_predict_covariance": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_int32, _VP, C.c_int64, C.c_int32, _VP]),
    "pgb_batch_create": (C.c_int, [C.POINTER(Desc), C.c_int32, C.POINTER(_VP)]),
    "pgb_batch_destroy": (C.c_int, [_VP]),
    "pgb_batch_layout": (C.c_int, [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "pgb_batch_objective": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_batch_value_and_grad": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_batch_set_enabled": (C.c_int, [_VP, _VP, _VP]),
    "pgb_batch_status": (C.c_int, [_VP, C.POINTER(Status), _VP]),
    "pgb_gp_desc": (C.c_int, [_VP, C.POINTER(Desc)]),
    "pgb_gp_set_near_depth": (C.c_int, [_VP, C.c_int32]),
    "pgb_batch_set_near_depth": (C.c_int, [_VP, C.POINTER(C.c_int32)]),
    "pgb_batch_size": (C.c_int, [_VP, C.POINTER(C.c_int32)]),
    "pgb_batch_desc": (C.c_int, [_VP, C.c_int32, C.POINTER(Desc)]),
    # include/probit_gb300_dlpack.h (DLTensor arguments as addresses)
    "pgb_dl_check": (C.c_int, [_VP, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int64), C.c_int32]),
    "pgb_dl_weight": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_dl_approximate_posterior": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_dl_objective": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_dl_value_and_grad": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_dl_vb_value_and_grad": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "pgb_dl_predict": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, C.c_int32, _VP]),
    "pgb_dl_batch_value_and_grad": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols() -> list[str]:
    """Names of the functions the C-ABI binding declares."""
    return list(_SIGS)


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the library once (raises ``NativeLibraryError`` if it is absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise NativeLibraryError(
                f"{p} not found: build it with `python -m probit_gb300.build` (nvcc, sm_103a)")
        try:
            lib = C.CDLL(str(p))
        except OSError as e:  # pragma: no cover - depends on the host
            raise NativeLibraryError(f"cannot load {p}: {e}") from e
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def strerror(code: int) -> str:
    try:
        return load().pgb_strerror(int(code)).decode()
    except NativeLibraryError:
        return f"error {code}"


def check(code: int, where: str) -> None:
    if code != PGB_OK:
        raise PgbError(code, where)
