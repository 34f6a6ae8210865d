"""The tensor-core tile product (tensor-map loads, in-place TF32 hi/lo split,
tcgen05 3xTF32 MMAs, TMEM read-back) against a float64 product.

C = A B^T for 128 x K operands; the 3xTF32 error bound is a few 2^-22 of
sum_k |a_k b_k| per entry, so the check is 2e-6 of that scale.
"""

import ctypes as C

import numpy as np
import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("K", [128, 512, 1024])
def test_tc_tile_product(native_lib, cuda_device, K):
    import torch

    lib = native_lib
    lib.pgbx_tc_tile_check.restype = C.c_int
    lib.pgbx_tc_tile_check.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((128, K)).astype(np.float32)
    Ad = torch.from_numpy(A).to(cuda_device)
    Bd = torch.from_numpy(B).to(cuda_device)
    Cd = torch.full((128, 128), float("nan"), dtype=torch.float32, device=cuda_device)
    st = torch.zeros(8, dtype=torch.int32, device=cuda_device)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.pgbx_tc_tile_check(Ad.data_ptr(), Bd.data_ptr(), K, Cd.data_ptr(), st.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert int(st[0]) == 0
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    err = np.abs(Cd.cpu().numpy() - ref) / scale
    assert np.isfinite(Cd.cpu().numpy()).all()
    assert err.max() < 2e-6, err.max()
