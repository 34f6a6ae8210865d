"""pgb_gram_noalloc against pgb_gram, through the C-ABI.

pgb_gram_noalloc exists for callers that cannot allocate device memory while
they run (an XLA FFI custom call inside JAX's preallocated pool, work recorded
by stream capture, services that reserve memory up front).  Its scratch is a
fixed array inside the library that every call shares, so these tests make
calls in a row with different shapes and kernels: a later call must not see
anything left over by an earlier one.  The scratch holds (n1 + n2) * ceil4(F)
floats, F the kernel's feature count (d, 2d for eq_periodic): a request that
fills it exactly is served, one more point is refused.

The file name sorts after every other test file, so a run that stops at the
first failure has run all other tests before these.
"""

import numpy as np
import pytest

from probit_gb300 import _native as N

SCRATCH_FLOATS = 1 << 20


def _dp(kernel, d):
    f = 2 * d if kernel == N.KERNEL_EQ_PERIODIC else d
    return (f + 3) // 4 * 4


def _gram(lib, fn, kernel, X1, X2, theta, ld):
    import torch

    n1, d = X1.shape
    n2 = X2.shape[0]
    desc = N.Desc(n1, d, kernel, d, 0.5, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
    x1 = torch.from_numpy(X1).cuda()
    x2 = torch.from_numpy(X2).cuda()
    th = torch.from_numpy(theta).cuda()
    K = torch.full((n1, ld), -7.0, device="cuda")
    rc = getattr(lib, fn)(desc, th.data_ptr(), x1.data_ptr(), n1, x2.data_ptr(), n2, K.data_ptr(), ld,
                          torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, K.cpu().numpy()


def _check_pair(lib, rng, kernel, n1, n2, d):
    X1 = rng.uniform(-2, 2, (n1, d)).astype(np.float32)
    X2 = rng.uniform(-2, 2, (n2, d)).astype(np.float32)
    ell = rng.uniform(0.5, 2.0, d)
    theta = np.array(list(ell) + [1.4, 0.1], dtype=np.float32)
    ld = n2 + 3
    rc_ref, K_ref = _gram(lib, "pgb_gram", kernel, X1, X2, theta, ld)
    rc, K = _gram(lib, "pgb_gram_noalloc", kernel, X1, X2, theta, ld)
    assert rc_ref == N.PGB_OK and rc == N.PGB_OK
    assert np.abs(K[:, :n2] - K_ref[:, :n2]).max() <= 1e-6
    assert (K[:, n2:] == -7.0).all()


@pytest.mark.gpu
def test_gram_noalloc_matches_gram_twice(native_lib, cuda_device):
    rng = np.random.default_rng(11)
    # a large request first, then a smaller one of another kernel and width
    _check_pair(native_lib, rng, N.KERNEL_EQ_PERIODIC, 300, 170, 3)
    _check_pair(native_lib, rng, N.KERNEL_MATERN12, 90, 250, 5)


@pytest.mark.gpu
@pytest.mark.parametrize("kernel,d", [(N.KERNEL_EQ, 4), (N.KERNEL_EQ_PERIODIC, 3)])
def test_gram_noalloc_at_its_scratch_limit(native_lib, cuda_device, kernel, d):
    """(n1 + n2) * ceil4(F) == 1,048,576: served and equal to pgb_gram, twice
    in a row; one point more: refused with PGB_EUNSUPPORTED before any launch.
    eq_periodic with d = 3 has F = 6 features (stride 8), so its limit is half
    that of a 4-feature EQ kernel."""
    import torch

    rng = np.random.default_rng(5 + d)
    dp = _dp(kernel, d)
    total = SCRATCH_FLOATS // dp
    n1 = 16
    _check_pair(native_lib, rng, kernel, n1, total - n1, d)
    _check_pair(native_lib, rng, kernel, n1 + 8, total - n1 - 8, d)
    desc = N.Desc(n1, d, kernel, d, 0.5, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
    buf = torch.zeros(8, device="cuda")
    rc = native_lib.pgb_gram_noalloc(desc, buf.data_ptr(), buf.data_ptr(), n1, buf.data_ptr(), total - n1 + 1,
                                     buf.data_ptr(), total - n1 + 1, None)
    assert rc == N.PGB_EUNSUPPORTED


@pytest.mark.gpu
def test_gram_noalloc_rejects_requests_beyond_its_scratch(native_lib, cuda_device):
    """300,000 points of 4 features need 1.2M scratch floats (> 1,048,576):
    refused on the host with PGB_EUNSUPPORTED before anything is launched."""
    import torch

    desc = N.Desc(200000, 4, N.KERNEL_EQ, 4, 1.0, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
    buf = torch.zeros(8, device="cuda")
    rc = native_lib.pgb_gram_noalloc(desc, buf.data_ptr(), buf.data_ptr(), 200000, buf.data_ptr(), 100000,
                                     buf.data_ptr(), 100000, None)
    assert rc == N.PGB_EUNSUPPORTED
