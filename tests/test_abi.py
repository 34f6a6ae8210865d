"""The C-ABI library loads and exports every function include/*.h declares."""

import ctypes as C
import re
from pathlib import Path

import pytest

from probit_gb300 import _native as N

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(pgb_[a-z_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_binding():
    assert declared_functions() == sorted(N.exported_symbols())


def test_library_exports_every_declared_symbol(native_lib):
    for name in declared_functions():
        assert hasattr(native_lib, name), name


def test_theta_size_and_validation(native_lib):
    d = N.Desc(100, 3, N.KERNEL_EQ, 3, 1.0, N.LIK_PROBIT, 5, 1e-5, 100, 0)
    assert native_lib.pgb_theta_size(d) == 3 + 2 + 6
    d.n_lengthscales = 1
    assert native_lib.pgb_theta_size(d) == 1 + 2 + 6
    d.likelihood = N.LIK_GAUSSIAN
    assert native_lib.pgb_theta_size(d) == 3
    for field, bad in (("n", 0), ("d", 17), ("kernel", 9), ("n_lengthscales", 2), ("maxiter", 0),
                       ("flags", 1)):
        e = N.Desc(100, 3, N.KERNEL_EQ, 1, 1.0, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
        setattr(e, field, bad)
        assert native_lib.pgb_theta_size(e) == N.PGB_EINVAL, field
    e = N.Desc(100, 1, N.KERNEL_EQ_PERIODIC, 1, 0.0, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
    assert native_lib.pgb_theta_size(e) == N.PGB_EINVAL
    # the periodic kernel uses two features (sin, cos) per input dimension
    e = N.Desc(100, 9, N.KERNEL_EQ_PERIODIC, 1, 0.5, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
    assert native_lib.pgb_theta_size(e) == N.PGB_EUNSUPPORTED
    e.d = 8
    assert native_lib.pgb_theta_size(e) == 3


def test_strerror_and_version(native_lib):
    assert b"sm_103a" in native_lib.pgb_version()
    assert native_lib.pgb_strerror(N.PGB_ENOTPD).decode().startswith("B = I")
    assert native_lib.pgb_strerror(12345) == b"unknown error"


def test_null_arguments_are_rejected(native_lib):
    assert native_lib.pgb_gp_create(None, None) == N.PGB_EINVAL
    assert native_lib.pgb_gp_destroy(None) == N.PGB_OK
    d = N.Desc(10, 2, N.KERNEL_EQ, 1, 1.0, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
    assert native_lib.pgb_gram(d, None, None, 1, None, 1, None, 1, None) == N.PGB_EINVAL
    assert native_lib.pgb_weight(None, None, None, None, None, None) == N.PGB_EINVAL
    assert native_lib.pgb_predict(None, None, None, None, None, None, 1, None, None, 0, None) == N.PGB_EINVAL
