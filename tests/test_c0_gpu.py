"""Config 0 end to end: the reference's ordinal classification example scaled
up (examples/classification.py:371-375) -- N = 512 points X ~ U[-2, 2]^2,
Matern12 (l = 1, s = 1), J = 3 classes at cutpoints (-0.5, 0.5), noise std
sqrt(0.4), predictions on a 40 x 25 grid (M = 1,000) -- through LaplaceGP at
the reference's default tolerance 1e-5 (approximators.py:62), against the
oracle's restatement of approximators.py:204-210 (approximate_posterior),
:265-277 (weight, precision), :154-180 (predict) and implicit/Laplace.py
(objective) in float64 and float32.

Bars: negative log evidence 1e-4 relative to the float64 and the float32
oracle; weight a and predictive mean 1e-4 of their largest magnitude; the
positive precision W and predictive variance 1e-4 relative, entry by entry;
the gradient 1e-3 of its largest entry.  Newton iterations within 1 of the
float64 oracle's or of the float32 oracle's: at tolerance 1e-5 the float32
restatement of the reference stalls at its rounding floor and runs to
maxiter = 100, while float64 converges in 5 steps.  The config's own rule,
||f_k - f_{k-1}|| < 1e-6, is evaluated on the GPU's last Newton update (f
follows a by f += K da) and reported beside the reference's ||a_k - a_{k-1}||.
"""

import ctypes as C

import numpy as np
import pytest

import probit_gb300 as pg
from oracle import laplace as L
from probit_gb300 import workloads as W

TOL = 1e-5


@pytest.fixture(scope="module")
def c0(cuda_device):
    p = W.ordinal_c0()
    op = L.Problem(p.X.astype(np.float64), p.y, "matern12", "probit", 1, 0.5, 3)
    th = p.theta()
    a64, it64 = L.newton_weight(op, th, tol=TOL)
    _, it32 = L.newton_weight(op, th.astype(np.float32), tol=TOL, dtype=np.float32)
    W64, f64 = L.precision(op, th, a64)
    v64, g64, _, _ = L.value_and_grad(op, th, tol=TOL)
    v32, _, _, _ = L.value_and_grad(op, th.astype(np.float32), tol=TOL, dtype=np.float32)
    m64, s64 = L.predict(op, th, p.Xtest.astype(np.float64), a64, W64)
    return p, dict(a=a64, W=W64, f=f64, it64=it64, it32=it32, v64=v64, v32=v32, g64=g64, mean=m64, var=s64)


@pytest.mark.gpu
def test_c0_posterior_evidence_and_predict(c0):
    p, ref = c0
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=TOL)
    params = p.params()
    a, Wp = gp.approximate_posterior(params)
    a, Wp = np.asarray(a, np.float64), np.asarray(Wp, np.float64)
    it = gp.last_status()[1]
    v, g = gp.value_and_grad()(params)
    mean, var = gp.predict(p.Xtest, params, a.astype(np.float32), Wp.astype(np.float32))
    mean, var = np.asarray(mean, np.float64), np.asarray(var, np.float64)
    gflat = np.array([g[0][0], g[0][1], g[1][0], *np.asarray(g[1][1])], np.float64)
    assert abs(v - ref["v64"]) <= 1e-4 * abs(ref["v64"]), (v, ref["v64"])
    assert abs(v - ref["v32"]) <= 1e-4 * abs(ref["v32"]), (v, ref["v32"])
    assert np.abs(a - ref["a"]).max() <= 1e-4 * np.abs(ref["a"]).max()
    assert (np.abs(Wp - ref["W"]) <= 1e-4 * ref["W"]).all()
    assert np.abs(mean - ref["mean"]).max() <= 1e-4 * np.abs(ref["mean"]).max()
    assert (np.abs(var - ref["var"]) <= 1e-4 * ref["var"]).all()
    g64 = ref["g64"]
    assert np.abs(gflat - g64).max() <= 1e-3 * np.abs(g64).max(), (gflat, g64)
    assert abs(it - ref["it64"]) <= 1 or abs(it - ref["it32"]) <= 1, (it, ref["it64"], ref["it32"])


@pytest.mark.gpu
def test_c0_config_stopping_rule(c0, native_lib):
    """||f_k - f_{k-1}|| = ||K da|| of the last Newton update, in float64 on
    the host from the GPU's da, reported beside ||da||, which the reference's
    rule (||da|| <= 1e-5, else maxiter) stopped the loop on."""
    import torch

    p, ref = c0
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=TOL)
    gp.approximate_posterior(p.params())
    torch.cuda.synchronize()
    native_lib.pgbx_gp_buffer.restype = C.c_void_p
    native_lib.pgbx_gp_buffer.argtypes = [C.c_void_p, C.c_char_p]
    handle = gp._last_handle
    ptr = native_lib.pgbx_gp_buffer(handle.h, b"da")
    n = p.N

    class _Dev:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False), "version": 2,
                                    "strides": None}

    da = torch.as_tensor(_Dev(), device="cuda").cpu().numpy().astype(np.float64)
    op = L.Problem(p.X.astype(np.float64), p.y, "matern12", "probit", 1, 0.5, 3)
    K = L._K(op, p.theta(), np.float64)
    dnorm, fnorm = np.linalg.norm(da), np.linalg.norm(K @ da)
    print(f"last Newton update: ||da|| = {dnorm:.3e}, ||K da|| = ||df|| = {fnorm:.3e}")
    assert dnorm <= TOL or gp.last_status()[1] >= 100
    assert np.isfinite(fnorm)
