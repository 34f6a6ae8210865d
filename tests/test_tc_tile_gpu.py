"""The tensor-core tile product (TF32 hi/lo splits loaded by tensor maps,
tcgen05 3xTF32 MMAs into partial accumulators folded into a running fp32
sum, TMEM read-back) against a float64 product.

C = A B^T for 128 x K operands; the 3xTF32 error bound is a few 2^-22 of
sum_k |a_k b_k| per entry, so the check is 2e-6 of that scale.  With
all-positive operands (the diagonal of a Cholesky update sums squares) the
errors must not share a sign: the mean signed error over the tile is a
bias the factorisation accumulates over its tile columns.
"""

import ctypes as C

import numpy as np
import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("K", [128, 512, 1024])
def test_tc_tile_product(native_lib, cuda_device, K):
    rng = np.random.default_rng(K)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((128, K)).astype(np.float32)
    _check(native_lib, cuda_device, A, B)


@pytest.mark.gpu
def test_tc_tile_product_has_no_bias(native_lib, cuda_device):
    """Sums of K = 8192 positive products (C_ij ~ K/4): the mean signed
    relative error stays below 1e-6.  Accumulating the whole k-range in one
    tensor-core accumulator, whose rounding leans one way by a fraction of
    its magnitude's ulp at every MMA, biases the diagonal of L by 2e-5 after
    64 tile columns of a factorisation; 128-wide partials leave -1.1e-6 here."""
    K = 8192
    rng = np.random.default_rng(K + 1)
    A = rng.uniform(0.0, 1.0, (128, K)).astype(np.float32)
    B = rng.uniform(0.0, 1.0, (128, K)).astype(np.float32)
    signed = _check(native_lib, cuda_device, A, B)
    assert abs(signed.mean()) < 1e-6, signed.mean()


def _check(lib, cuda_device, A, B):
    import torch

    K = A.shape[1]
    lib.pgbx_tc_tile_check.restype = C.c_int
    lib.pgbx_tc_tile_check.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
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
    got = Cd.cpu().numpy().astype(np.float64)
    signed = (got - ref) / scale
    assert np.isfinite(got).all()
    assert np.abs(signed).max() < 2e-6, np.abs(signed).max()
    return signed
