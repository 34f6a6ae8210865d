"""The oracle's Variational-Bayes restatement (VBGP, approximators.py:280-339;
implicit/VB.py) on the CPU: the fixed point property, the B-form of the
objective the CUDA path evaluates, and float32 against float64."""

import math

import numpy as np
import pytest

from oracle import laplace as L
from probit_gb300 import workloads as W


def _problem(seed, N, D, J, kind):
    rng = np.random.default_rng(seed)
    p = W.ordinal_problem(rng, N, D, J, kind, 0.8, 1.2, math.sqrt(0.4), list(np.linspace(-1.0, 1.0, J - 1)))
    return L.Problem(p.X.astype(np.float64), p.y, p.kernel, "probit", p.lengthscale.size, p.period, p.J), p.theta()


CASES = [(1, 40, 1, 3, "eq"), (2, 90, 2, 5, "matern12"), (3, 70, 3, 4, "eq_periodic")]


@pytest.mark.parametrize("seed,N,D,J,kind", CASES)
def test_vb_fixed_point(seed, N, D, J, kind):
    op, th = _problem(seed, N, D, J, kind)
    w, it = L.vb_weight(op, th, tol=1e-10)
    assert it < 100
    w2 = L.vb_map(op, th, w)
    assert np.abs(w2 - w).max() <= 1e-9 * max(1.0, np.abs(w).max())


@pytest.mark.parametrize("seed,N,D,J,kind", CASES)
def test_vb_objective_bform(seed, N, D, J, kind):
    """sum_i [rowdot_i / 2 sigma + (B^-1)_ii / 2 + m_i w_i / 2 + log L_ii - 1/2 - log p_i]
    with B = I + K / sigma^2 equals objective_VB term by term."""
    op, th = _problem(seed, N, D, J, kind)
    w, _ = L.vb_weight(op, th, tol=1e-8)
    a = L.vb_objective(op, th, w)
    b = L.vb_objective_bform(op, th, w)
    assert np.isfinite(a)
    assert abs(a - b) <= 1e-10 * abs(a)


def test_vb_float32_close_to_float64():
    op, th = _problem(5, 120, 2, 4, "eq")
    w64, _ = L.vb_weight(op, th, tol=1e-6)
    w32, _ = L.vb_weight(op, th, tol=1e-4, dtype=np.float32)
    assert np.abs(w32 - w64).max() <= 1e-3 * np.abs(w64).max()
    o64 = L.vb_objective(op, th, w64)
    o32 = L.vb_objective(op, th, w32, dtype=np.float32)
    assert abs(o32 - o64) <= 1e-4 * abs(o64)


@pytest.mark.parametrize("seed,N,D,J,kind", CASES)
def test_vb_gradient_matches_finite_differences(seed, N, D, J, kind):
    """The oracle's implicit-layer VB gradient (adjoint fixed point over f_VB)
    against central differences of objective_VB(theta, w*(theta)), float64."""
    op, th = _problem(seed, N, D, J, kind)
    th = th.astype(np.float64)
    _, g, _, _ = L.vb_value_and_grad(op, th, tol=1e-13, maxiter=5000)

    def F(t):
        w, _ = L.vb_weight(op, t, tol=1e-13, maxiter=5000)
        return L.vb_objective(op, t, w)

    for k in range(th.size):
        if not np.isfinite(th[k]):
            assert g[k] == 0.0
            continue
        h = 1e-5 * max(1.0, abs(th[k]))
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd = (F(tp) - F(tm)) / (2 * h)
        assert abs(g[k] - fd) <= 1e-6 * max(1.0, abs(fd)), (k, g[k], fd)
