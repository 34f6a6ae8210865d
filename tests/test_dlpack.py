"""DLPack entry points (include/probit_gb300_dlpack.h).

The library reads the DLTensor that torch's own DLPack producer writes
(pointer, device, dtype, shape, strides), and rejects wrong dtypes, shapes,
strides, devices and null handles before any CUDA call (CPU).  The GPU
check (DLPack and pointer calls give the same bits) is in
test_zz_interfaces_gpu.py.
"""

import ctypes as C

import pytest

from probit_gb300 import _native as N

FLOAT, INT = 2, 0


def shape_arg(*dims):
    return (C.c_int64 * max(1, len(dims)))(*dims)


def check(lib, obj, code, bits, dims, allow_host=1):
    cap, addr = N.dlpack_tensor(obj)
    rc = lib.pgb_dl_check(addr, code, bits, len(dims), shape_arg(*dims), allow_host)
    del cap
    return rc


def test_reads_torch_dltensor(native_lib):
    import torch

    t = torch.arange(15, dtype=torch.float32).reshape(5, 3)
    cap, addr = N.dlpack_tensor(t)
    d = N.DLTensor.from_address(addr)
    assert d.data + d.byte_offset == t.data_ptr()
    assert (d.device_type, d.ndim, d.dtype_code, d.dtype_bits, d.dtype_lanes) == (1, 2, FLOAT, 32, 1)
    assert [d.shape[0], d.shape[1]] == [5, 3]
    assert native_lib.pgb_dl_check(addr, FLOAT, 32, 2, shape_arg(5, 3), 1) == N.PGB_OK
    # any extent where the expected extent is negative
    assert native_lib.pgb_dl_check(addr, FLOAT, 32, 2, shape_arg(-1, 3), 1) == N.PGB_OK
    del cap


@pytest.mark.parametrize("case", ["dtype", "bits", "shape", "ndim", "strides", "host"])
def test_rejects_mismatch(native_lib, case):
    import torch

    t = torch.zeros((6, 4), dtype=torch.float32)
    want = dict(obj=t, code=FLOAT, bits=32, dims=(6, 4), allow_host=1)
    if case == "dtype":
        want["obj"] = t.to(torch.int32)
    elif case == "bits":
        want["obj"] = t.to(torch.float64)
    elif case == "shape":
        want["dims"] = (6, 5)
    elif case == "ndim":
        want["dims"] = (24,)
    elif case == "strides":
        want["obj"] = t.t()          # column-major view
        want["dims"] = (4, 6)
    elif case == "host":
        want["allow_host"] = 0       # CPU memory where device memory is required
    assert check(native_lib, **want) == N.PGB_EINVAL


def test_accepts_compact_views(native_lib):
    import torch

    t = torch.zeros((8, 4), dtype=torch.float32)
    assert check(native_lib, t[2:5], FLOAT, 32, (3, 4)) == N.PGB_OK        # row slice: compact
    assert check(native_lib, t[:, :1], FLOAT, 32, (8, 1)) == N.PGB_EINVAL  # column slice: strided
    assert check(native_lib, t[3], FLOAT, 32, (4,)) == N.PGB_OK
    assert check(native_lib, torch.zeros(5, dtype=torch.int32), INT, 32, (5,)) == N.PGB_OK
    assert check(native_lib, torch.zeros((), dtype=torch.float32), FLOAT, 32, ()) == N.PGB_OK


def test_cuda_typed_tensor_passes_the_host_side_check(native_lib):
    # a descriptor that claims CUDA memory; pgb_dl_check reads only the
    # descriptor, never the memory
    shape = (C.c_int64 * 2)(7, 2)
    d = N.DLTensor(data=4096, device_type=2, device_id=0, ndim=2, dtype_code=FLOAT, dtype_bits=32,
                   dtype_lanes=1, shape=shape, strides=None, byte_offset=0)
    assert native_lib.pgb_dl_check(C.addressof(d), FLOAT, 32, 2, shape_arg(7, 2), 0) == N.PGB_OK
    d.byte_offset = 2   # start not 4-byte aligned
    assert native_lib.pgb_dl_check(C.addressof(d), FLOAT, 32, 2, shape_arg(7, 2), 0) == N.PGB_EINVAL
    d.byte_offset = 0
    d.dtype_lanes = 2
    assert native_lib.pgb_dl_check(C.addressof(d), FLOAT, 32, 2, shape_arg(7, 2), 0) == N.PGB_EINVAL


def test_null_handles_are_rejected(native_lib):
    assert native_lib.pgb_dl_value_and_grad(None, None, None, None, None, None, None) == N.PGB_EINVAL
    assert native_lib.pgb_dl_weight(None, None, None, None, None, None) == N.PGB_EINVAL
    assert native_lib.pgb_dl_predict(None, None, None, None, None, None, None, None, 0, None) == N.PGB_EINVAL
    assert native_lib.pgb_dl_batch_value_and_grad(None, None, None, None, None, None, None) == N.PGB_EINVAL
    assert native_lib.pgb_dl_check(None, FLOAT, 32, 0, None, 1) == N.PGB_EINVAL
    assert native_lib.pgb_gp_desc(None, None) == N.PGB_EINVAL
    assert native_lib.pgb_batch_size(None, None) == N.PGB_EINVAL
