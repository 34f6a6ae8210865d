"""pgb_gram_noalloc against pgb_gram, through the C-ABI.

pgb_gram_noalloc exists for callers that cannot allocate device memory while
they run (an XLA FFI custom call inside JAX's preallocated pool, work recorded
by stream capture, services that reserve memory up front).  Its scratch is a
fixed array inside the library that every call shares, so this test makes two
calls in a row with different shapes and kernels: the second must not see
anything left over by the first.  This file is collected last on purpose.
"""

import numpy as np
import pytest

from probit_gb300 import _native as N


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


@pytest.mark.gpu
def test_gram_noalloc_matches_gram_twice(native_lib, cuda_device):
    rng = np.random.default_rng(11)
    calls = [
        (N.KERNEL_EQ_PERIODIC, rng.uniform(-2, 2, (300, 3)), rng.uniform(-2, 2, (170, 3)), [0.7, 1.1, 1.6]),
        (N.KERNEL_MATERN12, rng.uniform(-2, 2, (90, 5)), rng.uniform(-2, 2, (250, 5)), [0.5, 0.8, 1.0, 1.3, 2.0]),
    ]
    for kernel, X1, X2, ell in calls:
        X1 = X1.astype(np.float32)
        X2 = X2.astype(np.float32)
        theta = np.array(list(ell) + [1.4, 0.1], dtype=np.float32)
        ld = X2.shape[0] + 3
        rc_ref, K_ref = _gram(native_lib, "pgb_gram", kernel, X1, X2, theta, ld)
        rc, K = _gram(native_lib, "pgb_gram_noalloc", kernel, X1, X2, theta, ld)
        assert rc_ref == N.PGB_OK and rc == N.PGB_OK
        n2 = X2.shape[0]
        assert np.abs(K[:, :n2] - K_ref[:, :n2]).max() <= 1e-6
        assert (K[:, n2:] == -7.0).all()


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
