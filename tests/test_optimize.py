"""Lockstep L-BFGS (probit_gb300.optimize) on the CPU."""

import numpy as np
import pytest

from probit_gb300.optimize import LogParams, minimize_lockstep


def _quadratics(B=6, P=5, seed=0):
    rng = np.random.default_rng(seed)
    As, bs = [], []
    for b in range(B):
        Q, _ = np.linalg.qr(rng.standard_normal((P, P)))
        ev = np.logspace(0, b % 4, P)           # condition numbers 1 .. 1e3
        As.append(Q @ np.diag(ev) @ Q.T)
        bs.append(rng.standard_normal(P))
    A, bv = np.array(As), np.array(bs)

    def fg(X, mask=None):
        AX = np.einsum("bij,bj->bi", A, X)
        return 0.5 * np.einsum("bi,bi->b", X, AX) - np.einsum("bi,bi->b", bv, X), AX - bv

    xstar = np.array([np.linalg.solve(a, v) for a, v in zip(A, bv)])
    return fg, xstar


def _rosenbrock(X, mask=None):
    a, b = X[:, 0], X[:, 1]
    f = (1 - a) ** 2 + 100 * (b - a * a) ** 2
    g = np.stack([-2 * (1 - a) - 400 * a * (b - a * a), 200 * (b - a * a)], axis=1)
    return f, g


def test_quadratics_converge():
    fg, xstar = _quadratics()
    res = minimize_lockstep(fg, np.zeros_like(xstar), maxiter=100, gtol=1e-9, ftol=0.0)
    assert res.converged.all()
    assert np.abs(res.x - xstar).max() < 1e-6


def test_rosenbrock_matches_scipy():
    scipy_opt = pytest.importorskip("scipy.optimize")
    x0 = np.array([[-1.2, 1.0], [0.5, -0.3], [2.0, 2.0]])
    res = minimize_lockstep(_rosenbrock, x0, maxiter=200, gtol=1e-8, ftol=0.0, max_ls=30)
    for b in range(3):
        ref = scipy_opt.minimize(lambda z: _rosenbrock(z[None])[0][0], x0[b], jac=lambda z: _rosenbrock(z[None])[1][0],
                                 method="L-BFGS-B", options={"gtol": 1e-10, "ftol": 1e-15, "maxiter": 500})
        assert np.allclose(res.x[b], ref.x, atol=1e-5)
        assert np.allclose(res.x[b], [1.0, 1.0], atol=1e-5)


def test_each_problem_moves_as_if_alone():
    """Lockstep evaluation does not couple problems: same iterates alone and together."""
    x0 = np.array([[-1.2, 1.0], [0.5, -0.3], [2.0, 2.0], [0.0, 0.0]])
    together = minimize_lockstep(_rosenbrock, x0, maxiter=25)
    for b in range(x0.shape[0]):
        alone = minimize_lockstep(_rosenbrock, x0[b:b + 1], maxiter=25)
        assert np.array_equal(alone.x[0], together.x[b])
        assert alone.iterations[0] == together.iterations[b]


def test_nonfinite_values_shorten_the_step():
    def fg(X, mask=None):
        f = np.where(X[:, 0] > 1.5, np.nan, (X[:, 0] - 1.0) ** 2)
        return f, np.stack([2 * (X[:, 0] - 1.0)], axis=1)

    res = minimize_lockstep(fg, np.array([[-3.0]]), maxiter=30, gtol=1e-10, ftol=0.0)
    assert abs(res.x[0, 0] - 1.0) < 1e-6


def test_logparams_roundtrip_and_chain_rule():
    lp = LogParams(nl=3, J=5)
    rng = np.random.default_rng(1)
    u = rng.normal(size=(4, 9))          # any u: the cutpoints come out ordered
    th = lp.to_theta(u)
    assert th.shape == (4, 3 + 2 + 6)
    assert np.isneginf(th[:, 5]).all() and np.isposinf(th[:, -1]).all()
    assert (np.diff(th[:, 6:10], axis=1) > 0).all()
    assert np.allclose(lp.from_theta(th), u)
    # d/du of h(theta(u)) for h(theta) = sum(w * finite theta) by central differences
    w = rng.normal(size=th.shape[1])
    fin = np.isfinite(th[0])

    def h(uu):
        t = lp.to_theta(uu)[0]
        return float(np.sum(w[fin] * t[fin]))

    gtheta = np.where(fin, w, 0.0)[None]
    gu = lp.grad_u(th[:1], gtheta)[0]
    eps = 1e-6
    fd = np.array([(h(u[:1] + eps * np.eye(9)[k]) - h(u[:1] - eps * np.eye(9)[k])) / (2 * eps) for k in range(9)])
    assert np.allclose(gu, fd, rtol=1e-6, atol=1e-8)


def test_logparams_binary_and_extreme_coordinates():
    lp = LogParams(nl=1, J=2)
    th = lp.to_theta(np.array([[0.1, -0.2, 0.3, 0.7]]))
    assert th.shape == (1, 1 + 2 + 3) and th[0, 4] == 0.7
    with np.errstate(over="raise", invalid="raise"):
        big = LogParams(nl=1, J=5).to_theta(np.array([[500.0, -500.0, 90.0, 1.0, 200.0, -300.0, 0.0]]))
    assert np.isfinite(big[:, :3]).all() and np.isfinite(big[:, 4:8]).all()
    assert np.isfinite(big.astype(np.float32)[:, :3]).all()
    with pytest.raises(ValueError):
        LogParams(nl=1, J=4).from_theta(np.array([[1.0, 1.0, 1.0, -np.inf, 0.5, 0.2, 0.9, np.inf]]))


def test_trial_steps_are_capped():
    """A long L-BFGS direction (a shallow slope beside a steep valley) moves
    no coordinate by more than max_step from the point its line search
    starts at, on any trial."""
    log = []

    def fg(X, mask=None):
        log.append(("eval", X.copy()))
        f = 1e-4 * X[:, 0] + 0.5 * X[:, 1] ** 2
        return f, np.stack([np.full(X.shape[0], 1e-4), X[:, 1]], axis=1)

    x0 = np.array([[0.0, 1e-3]])
    minimize_lockstep(fg, x0, maxiter=6, max_step=0.5, ftol=0.0, gtol=0.0,
                      callback=lambda x, f, g: log.append(("acc", x.copy())))
    base, trials = x0, 0
    for kind, x in log[1:]:
        if kind == "acc":
            base = x
        else:
            assert np.abs(x - base).max() <= 0.5 + 1e-12
            trials += 1
    assert trials >= 6
    # without the cap the first direction (gamma = 1 / ||g||) would move ~1
    assert np.abs(log[1][1] - x0).max() == pytest.approx(0.5)
