"""Full-size parity: the N = 8192 evidence + gradient and M = 65,536 predict
workloads (Gaussian
likelihood, EQ with four lengthscales, D = 4, the benchmark's problem)
against a size-independent property.  For a Gaussian likelihood the Laplace
evidence is the exact GP marginal likelihood

    -log Z = 1/2 y^T C^-1 y + sum log diag chol(C) + N/2 log 2 pi,   C = K + sigma^2 I,

with gradient 1/2 tr(C^-1 dK) - 1/2 alpha^T dK alpha (alpha = C^-1 y) for
the kernel's parameters and sigma tr(C^-1) - sigma alpha^T alpha for the
noise std, evaluated here in float64.  Bars: the log evidence to 1e-4
relative; the gradient to 1e-2 of its largest component (its entries are
differences of O(N) terms near the generating hyperparameters).  The
closed form itself is checked against the oracle on the CPU at N = 300.

Collected after the other GPU tests: the float64 reference (a Cholesky and
an inverse of an 8192 x 8192 matrix) takes tens of seconds on the host.
"""

import math

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import laplace as L


def exact_gaussian(X, y, theta, nl, block=1024):
    """(-log Z, gradient) of the exact marginal likelihood, float64."""
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    ell, s, sig = theta[:nl], float(theta[nl]), float(theta[nl + 1])
    n = X.shape[0]
    C = L.gram("eq", X, X, ell, s)
    C[np.diag_indices(n)] += sig * sig
    cf = sla.cho_factor(C, lower=True, overwrite_a=True, check_finite=False)
    alpha = sla.cho_solve(cf, y, check_finite=False)
    value = 0.5 * y @ alpha + np.log(np.diag(cf[0])).sum() + 0.5 * n * math.log(2 * math.pi)
    Cinv = sla.cho_solve(cf, np.eye(n), overwrite_b=True, check_finite=False)
    grad = np.zeros(nl + 2)
    for r0 in range(0, n, block):
        rows = slice(r0, min(n, r0 + block))
        _, dKs = L.gram_param_derivs("eq", X, ell, s, rows=rows)
        for k, dK in enumerate(dKs):
            grad[k] += 0.5 * np.sum(Cinv[rows] * dK) - 0.5 * alpha[rows] @ (dK @ alpha)
    grad[nl + 1] = sig * np.trace(Cinv) - sig * alpha @ alpha
    return value, grad


def test_closed_form_matches_oracle():
    from probit_gb300 import workloads as W

    p = W.regression_problem(np.random.default_rng(5), 300, 4, "eq", [0.5, 1.0, 1.5, 2.0], 1.0, 0.2)
    theta = p.theta()
    v, g = exact_gaussian(p.X, p.y, theta, 4)
    op = L.Problem(np.asarray(p.X, np.float64), np.asarray(p.y, np.float64), "eq", "gaussian", 4)
    v64, g64, _, _ = L.value_and_grad(op, theta, tol=1e-10)
    assert abs(v - v64) <= 1e-10 * abs(v64)
    assert np.allclose(g, g64, rtol=1e-7, atol=1e-8)


@pytest.mark.gpu
def test_n8192_evidence_and_gradient(cuda_device):
    import probit_gb300 as pg
    from probit_gb300 import workloads as W

    p = W.regression_c1(N=8192, M=0)   # the benchmark's problem (host draw)
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_gaussian_likelihood, tolerance=1.0)
    v, g = gp.value_and_grad()(p.params())
    g = np.concatenate([np.ravel(np.asarray(g[0][0], np.float64)), [float(g[0][1])], [float(g[1][0])]])
    v64, g64 = exact_gaussian(p.X, p.y, p.theta(), 4)
    assert abs(float(v) - v64) <= 1e-4 * abs(v64), (float(v), v64)
    assert np.abs(g - g64).max() <= 1e-2 * np.abs(g64).max(), (g, g64)


@pytest.mark.gpu
def test_n8192_predict_m65536(cuda_device):
    """Predictive mean and variance at the benchmark's 65,536 test points
    against the Gaussian closed form (mean K_*^T C^-1 y, variance
    s - diag(K_*^T C^-1 K_*)) in float64 at every 64th point: the mean to
    1e-4 of its largest magnitude, the variance to 1e-4 of the signal
    variance s."""
    import probit_gb300 as pg
    from probit_gb300 import workloads as W

    p = W.regression_c1(N=8192, M=65536)
    params = p.params()
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_gaussian_likelihood, tolerance=1.0)
    a, Wp = gp.approximate_posterior(params)
    mean, var = gp.predict(p.Xtest, params, a, Wp)
    assert mean.shape == (65536,) and var.shape == (65536,)
    th = p.theta()
    ell, s, sig = th[:4], float(th[4]), float(th[5])
    X = np.asarray(p.X, np.float64)
    Xs = np.asarray(p.Xtest, np.float64)[::64]
    C = L.gram("eq", X, X, ell, s)
    C[np.diag_indices(X.shape[0])] += sig * sig
    cf = sla.cho_factor(C, lower=True, overwrite_a=True, check_finite=False)
    Ks = L.gram("eq", X, Xs, ell, s)
    m64 = Ks.T @ sla.cho_solve(cf, np.asarray(p.y, np.float64), check_finite=False)
    V = sla.solve_triangular(cf[0], Ks, lower=True, check_finite=False)
    v64 = s - np.einsum("ij,ij->j", V, V)
    m, v = np.asarray(mean, np.float64)[::64], np.asarray(var, np.float64)[::64]
    assert np.abs(m - m64).max() <= 1e-4 * np.abs(m64).max(), np.abs(m - m64).max()
    assert np.abs(v - v64).max() <= 1e-4 * s, np.abs(v - v64).max()
