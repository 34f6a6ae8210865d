"""VBGP through the C-ABI (pgb_vb_weight, pgb_vb_objective,
pgb_vb_value_and_grad) against the float64 oracle restatement of VBGP
(approximators.py:280-339, implicit/VB.py): the fixed point to 1e-3 of its
largest entry, the objective to 1e-4 relative, the iteration count within 2
of the interval spanned by the oracle's float32 and float64 counts (the VB map
contracts slowly, by ~0.8 a step on the N = 513 case, so near the 1e-4
tolerance float32 rounding moves the count: the oracle takes 50 steps in
float32 and 40 in float64 there), the gradient to 1e-3 of its largest entry, and predictions
with the VB precision 1 / sigma^2 against the oracle's Approximator.predict."""

import math

import numpy as np
import pytest

import probit_gb300 as pg
from oracle import laplace as L
from probit_gb300 import workloads as W

CASES = [(11, 60, 1, 3, "eq"), (12, 129, 2, 5, "matern12"), (13, 300, 3, 4, "eq_periodic"), (14, 513, 2, 6, "eq")]
TOL = 1e-4


def _setup(seed, N, D, J, kind):
    rng = np.random.default_rng(seed)
    p = W.ordinal_problem(rng, N, D, J, kind, 0.8, 1.2, math.sqrt(0.4), list(np.linspace(-1.0, 1.0, J - 1)))
    op = L.Problem(p.X.astype(np.float64), p.y, p.kernel, "probit", p.lengthscale.size, p.period, p.J)
    gp = pg.VBGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=TOL)
    return p, op, gp


@pytest.mark.gpu
@pytest.mark.parametrize("seed,N,D,J,kind", CASES)
def test_vb_weight_and_objective(cuda_device, seed, N, D, J, kind):
    p, op, gp = _setup(seed, N, D, J, kind)
    params = p.params()
    w = np.asarray(gp.weight(params), np.float64)
    it = gp.last_status()[1]
    w64, it64 = L.vb_weight(op, p.theta(), tol=TOL)
    _, it32 = L.vb_weight(op, p.theta(), tol=TOL, dtype=np.float32)
    assert np.abs(w - w64).max() <= 1e-3 * np.abs(w64).max(), (np.abs(w - w64).max(), np.abs(w64).max())
    assert min(it32, it64) - 2 <= it <= max(it32, it64) + 2, (it, it32, it64)
    v = gp.objective()(params)
    v64 = L.vb_objective(op, p.theta(), w64)
    assert abs(v - v64) <= 1e-4 * abs(v64), (v, v64)


@pytest.mark.gpu
@pytest.mark.parametrize("seed,N,D,J,kind", CASES)
def test_vb_value_and_grad(cuda_device, seed, N, D, J, kind):
    p, op, gp = _setup(seed, N, D, J, kind)
    params = p.params()
    v, g = gp.value_and_grad()(params)
    from probit_gb300.approximators import tree_leaves

    gf = np.concatenate([np.atleast_1d(np.asarray(x, np.float64)) for x in tree_leaves(g)])
    v64, g64, _, _ = L.vb_value_and_grad(op, p.theta(), tol=TOL)
    assert abs(v - v64) <= 1e-4 * abs(v64), (v, v64)
    assert np.abs(gf - g64).max() <= 1e-3 * np.abs(g64).max(), (gf, g64)
    assert abs(gp.objective()(params) - v) <= 1e-6 * abs(v)


@pytest.mark.gpu
def test_vb_predict(cuda_device):
    p, op, gp = _setup(15, 200, 2, 4, "eq")
    params = p.params()
    w, Wp = gp.approximate_posterior(params)
    sig = math.sqrt(0.4)
    assert np.allclose(np.asarray(Wp), 1.0 / sig ** 2)
    Xs = np.random.default_rng(16).uniform(-2, 2, size=(97, 2)).astype(np.float32)
    mean, var = gp.predict(Xs, params, w, Wp)
    m64, v64 = L.predict(op, p.theta(), Xs.astype(np.float64), np.asarray(w, np.float64), np.asarray(Wp, np.float64))
    assert np.abs(np.asarray(mean) - m64).max() <= 1e-4 * max(1.0, np.abs(m64).max())
    assert np.abs(np.asarray(var) - v64).max() <= 1e-4 * max(1.0, np.abs(v64).max())


@pytest.mark.gpu
def test_vb_and_laplace_share_a_handle(cuda_device):
    """VB and Laplace operations interleaved on one native handle give the
    same bits as each alone (the VB factor is never taken for a Laplace one)."""
    p, op, gp = _setup(17, 150, 2, 3, "matern12")
    params = p.params()
    laplace = pg.LaplaceGP.objective(gp)   # the base class's objective on the same handles
    v1 = laplace(params)
    vb1 = gp.objective()(params)
    v2 = laplace(params)
    gp.weight(params)
    vb2 = gp.objective()(params)
    v3 = laplace(params)
    assert v1 == v2 == v3
    assert vb1 == vb2
    lap = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=TOL)
    assert lap.objective()(params) == v1
