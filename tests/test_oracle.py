"""The CPU oracle against the reference's known answers and analytic identities."""

import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import laplace as L

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
from cases import CASES, make, oracle_problem  # noqa: E402


def test_h_matches_reference_known_answers():
    """probit/test/test_implicit.py:11-22 (values of the tail polynomial h)."""
    with np.errstate(all="ignore"):
        assert np.isnan(L.h(0.0))
        assert L.h(np.inf) == 0.0
        assert L.h(-np.inf) == 0.0
    assert np.isclose(L.h(1.0), -65 / 6, rtol=1e-12)
    # its derivative: NaN at 0 and 0 at +-inf (central difference away from 0)
    x = 3.0
    d = (L.h(x + 1e-6) - L.h(x - 1e-6)) / 2e-6
    assert np.isclose(d, 2 * x ** -3 - 10 * x ** -5 + 74 * x ** -7, rtol=1e-6)


def _small(kind, lik, N=40, D=2, nl=1, J=3, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-2, 2, size=(N, D))
    ell = np.full(nl, 0.8)
    K = L.gram(kind, X, X, ell, 1.0) + 1e-6 * np.eye(N)
    f = np.linalg.cholesky(K) @ rng.standard_normal(N)
    if lik == "gaussian":
        prob = L.Problem(X, f + 0.3 * rng.standard_normal(N), kind, lik, nl, 0.5, 0)
        theta = np.concatenate([ell * 1.1, [0.9, 0.3]])
    else:
        cut = np.array([-np.inf, -0.5, 0.5, np.inf])
        y = np.searchsorted(cut[1:-1], f + np.sqrt(0.4) * rng.standard_normal(N))
        prob = L.Problem(X, y, kind, lik, nl, 0.5, J)
        theta = np.concatenate([ell * 1.1, [0.9, np.sqrt(0.4)], cut])
    return prob, theta


@pytest.mark.parametrize("kind", L.KERNELS)
@pytest.mark.parametrize("lik", L.LIKELIHOODS)
@pytest.mark.parametrize("nl", [1, 2])
def test_implicit_gradient_matches_finite_differences(kind, lik, nl):
    prob, theta = _small(kind, lik, nl=nl)
    _, g, _, _ = L.value_and_grad(prob, theta, tol=1e-12)
    for k in range(theta.size):
        if not np.isfinite(theta[k]):
            assert g[k] == 0.0
            continue
        h = 1e-5
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (L.objective(prob, tp, tol=1e-13)[0] - L.objective(prob, tm, tol=1e-13)[0]) / (2 * h)
        assert abs(g[k] - fd) <= 1e-6 * max(1.0, np.abs(g).max()), (k, g[k], fd)


def test_gaussian_evidence_is_exact_marginal_likelihood():
    prob, theta = _small("eq", "gaussian", N=50)
    v = L.objective(prob, theta, tol=1e-12)[0]
    ell, s, sig, _ = prob.split(theta)
    K = L.gram("eq", prob.X, prob.X, ell, s) + sig ** 2 * np.eye(50)
    c = np.linalg.cholesky(K)
    exact = 0.5 * prob.y @ np.linalg.solve(K, prob.y) + np.log(np.diag(c)).sum() + 25 * np.log(2 * np.pi)
    assert abs(v - exact) < 1e-9 * abs(exact)


@pytest.mark.parametrize("kind", L.KERNELS)
def test_gaussian_prediction_is_exact_gp_posterior(kind):
    """With a Gaussian likelihood the Laplace approximation is exact: the
    weight is (K + s^2 I)^-1 y, W = 1/s^2, and predict / predict_covariance
    are the GP posterior mean, variance and covariance (computed here with a
    Cholesky solve, independently of the oracle's own formulas)."""
    prob, theta = _small(kind, "gaussian", N=60)
    ell, s, sig, _ = prob.split(theta)
    rng = np.random.default_rng(3)
    Xs = rng.uniform(-2.5, 2.5, size=(25, prob.X.shape[1]))
    a, _ = L.newton_weight(prob, theta, tol=1e-12)
    W, _ = L.precision(prob, theta, a)
    Kxx = L.gram(kind, prob.X, prob.X, ell, s, prob.period) + sig ** 2 * np.eye(60)
    Kxs = L.gram(kind, prob.X, Xs, ell, s, prob.period)
    Kss = L.gram(kind, Xs, Xs, ell, s, prob.period)
    c = np.linalg.cholesky(Kxx)
    alpha = np.linalg.solve(c.T, np.linalg.solve(c, prob.y))
    V = np.linalg.solve(c, Kxs)
    assert np.abs(a - alpha).max() <= 1e-9 * np.abs(alpha).max()
    assert np.allclose(W, 1.0 / sig ** 2, rtol=1e-12)
    mean, var = L.predict(prob, theta, Xs, a, W)
    assert np.abs(mean - Kxs.T @ alpha).max() <= 1e-9 * np.abs(mean).max()
    assert np.abs(var - (np.diag(Kss) - (V * V).sum(0))).max() <= 1e-9 * s
    cov = L.predict_covariance(prob, theta, Xs, a, W)
    assert np.abs(cov - (Kss - V.T @ V)).max() <= 1e-9 * s


@pytest.mark.parametrize("kind", L.KERNELS)
@pytest.mark.parametrize("lik", ["gaussian", "probit", "probit_stable"])
def test_bform_equals_reference_form(kind, lik):
    prob, theta = _small(kind, lik, N=60, seed=3)
    a, it = L.newton_weight(prob, theta, tol=1e-12)
    ab, itb = L.newton_weight_bform(prob, theta, tol=1e-12)
    assert it == itb
    assert np.abs(a - ab).max() < 1e-10 * max(1, np.abs(a).max())
    v = L.objective(prob, theta, a=a)[0]
    assert abs(v - L.objective_bform(prob, theta, a)) < 1e-10 * abs(v)


def test_stable_and_reference_probit_agree_in_the_bulk():
    f = np.linspace(-1.5, 1.5, 31)
    y = np.array([i % 3 for i in range(31)])
    cut = np.array([-np.inf, -0.5, 0.5, np.inf])
    r = L.lik_terms("probit", f, y, 0.6, cut)
    s = L.lik_terms("probit_stable", f, y, 0.6, cut)
    # the +1e-10 of the reference form shifts points with small P, most visibly
    # in d3, whose terms cancel to a small value
    for k, rtol in (("logp", 1e-6), ("d1", 1e-6), ("d2", 1e-5), ("d3", 1e-3)):
        assert np.allclose(r[k], s[k], rtol=rtol, atol=1e-8), k


def test_stable_probit_is_finite_in_far_tails():
    f = np.array([40.0, -40.0, 80.0])
    y = np.array([0, 2, 0])
    cut = np.array([-np.inf, -0.5, 0.5, np.inf])
    s = L.lik_terms("probit_stable", f, y, 0.5, cut, np.float32)
    assert all(np.isfinite(s[k]).all() for k in ("logp", "d1", "d2"))
    # the reference form floors at log(1e-10) there
    r = L.lik_terms("probit", f, y, 0.5, cut, np.float32)
    assert np.allclose(r["logp"], np.log(np.float32(1e-10)), rtol=1e-5)


@pytest.mark.parametrize("name", list(CASES))
def test_golden_fixtures_reproduce(name):
    """The committed fixtures are what the oracle computes today."""
    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    assert np.array_equal(g["X"], p.X) and np.array_equal(g["y"], p.y)
    op = oracle_problem(p, CASES[name][1])
    v, grad, a, it = L.value_and_grad(op, theta, tol=tol, dtype=np.float64)
    assert it == int(g["iters_f64"])
    assert np.allclose(a, g["a_f64"], rtol=1e-9, atol=1e-12)
    assert np.isclose(v, g["value_f64"], rtol=1e-10)
    assert np.allclose(grad, g["grad_f64"], rtol=1e-8, atol=1e-10)
    # float32 and float64 oracle runs agree to the parity bar
    assert abs(g["value_f32"] - g["value_f64"]) <= 1e-4 * abs(g["value_f64"])
    assert int(g["iters_f32"]) == int(g["iters_f64"])


def test_predictive_distributions_sum_to_one():
    mean = np.linspace(-2, 2, 7)
    var = np.full(7, 0.3)
    p = L.predictive_distributions(0.5, [-np.inf, -0.5, 0.5, np.inf], mean, var)
    assert np.allclose(p.sum(axis=1), 1.0)
