"""CUDA path vs the CPU oracle on the golden cases (through the C-ABI).

Bars (the parity contract): negative log evidence within 1e-4 relative of the
float32 oracle; weight, precision and predictive mean within 1e-4 of the
largest entry; predictive variance within 1e-4 of the signal variance;
gradient within 1e-3 of its largest entry; Newton iterations within 1.  Each
output's error against the float64 oracle is checked to the same bars, and
entry by entry (test_elementwise_relative).
"""

import sys
from pathlib import Path

import numpy as np
import pytest

import probit_gb300 as pg
from probit_gb300 import _native as N
from probit_gb300.approximators import tree_leaves

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
from cases import CASES, make  # noqa: E402

LIK = {"gaussian": pg.log_gaussian_likelihood, "probit": pg.log_probit_likelihood,
       "probit_stable": pg.log_probit_likelihood_stable}


def rel_max(x, ref):
    x, ref = np.asarray(x, np.float64), np.asarray(ref, np.float64)
    return float(np.abs(x - ref).max() / max(np.abs(ref).max(), 1e-30))


def flat(tree):
    return np.concatenate([np.atleast_1d(np.asarray(v, np.float64)) for v in tree_leaves(tree)])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_laplace_parity(name, cuda_device):
    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    lik = CASES[name][1]
    gp = pg.LaplaceGP((g["X"], g["y"]), p.prior(), LIK[lik], tolerance=tol)
    params = p.params()

    a, W = gp.approximate_posterior(params)
    code, iters, _, _ = gp.last_status()
    assert code == 0
    assert abs(iters - int(g["iters_f32"])) <= 1, (iters, int(g["iters_f32"]))
    for tag in ("f32", "f64"):
        assert rel_max(a, g[f"a_{tag}"]) < 1e-4, (tag, rel_max(a, g[f"a_{tag}"]))
        assert rel_max(W, g[f"W_{tag}"]) < 1e-4, (tag, rel_max(W, g[f"W_{tag}"]))

    value, grads = gp.value_and_grad()(params)
    gf = flat(grads)
    for tag in ("f32", "f64"):
        ref = float(g[f"value_{tag}"])
        assert abs(value - ref) <= 1e-4 * abs(ref), (tag, value, ref)
        gr = np.asarray(g[f"grad_{tag}"], np.float64)
        assert np.abs(gf - gr).max() <= 1e-3 * np.abs(gr).max(), (tag, gf, gr)
    assert gp.objective()(params) == pytest.approx(value, rel=1e-6)

    mean, var = gp.predict(g["Xtest"], params, a, W)
    s = p.variance
    for tag in ("f32", "f64"):
        assert rel_max(mean, g[f"mean_{tag}"]) < 1e-4, (tag, rel_max(mean, g[f"mean_{tag}"]))
        assert np.abs(var - g[f"var_{tag}"]).max() < 1e-4 * s, (tag, np.abs(var - g[f"var_{tag}"]).max())
    # the same prediction with the factor rebuilt from W (no resident factor)
    mean2, var2 = gp.predict(g["Xtest"], params, np.array(a), np.array(W))
    assert np.abs(mean2 - mean).max() <= 1e-6 * np.abs(mean).max()
    assert np.abs(var2 - var).max() <= 1e-5 * s


def rel_elem(x, ref, floor=0.0):
    """Largest element-wise relative error, each entry's denominator at least
    `floor` times the largest reference entry (for outputs that cross 0)."""
    x, ref = np.asarray(x, np.float64), np.asarray(ref, np.float64)
    den = np.maximum(np.abs(ref), floor * np.abs(ref).max() + 1e-30)
    return float((np.abs(x - ref) / den).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_elementwise_relative(name, cuda_device):
    """Entry by entry against the float64 oracle: the precision W (positive)
    within 1e-4 relative of every entry; the weights a and the predictive mean
    (which cross zero) within 1e-3 relative with denominators of at least 1%
    of the largest entry; the predictive variance within 1e-3 relative."""
    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    gp = pg.LaplaceGP((g["X"], g["y"]), p.prior(), LIK[CASES[name][1]], tolerance=tol)
    params = p.params()
    a, W = gp.approximate_posterior(params)
    mean, var = gp.predict(g["Xtest"], params, a, W)
    assert rel_elem(W, g["W_f64"]) < 1e-4, rel_elem(W, g["W_f64"])
    assert rel_elem(a, g["a_f64"], 1e-2) < 1e-3, rel_elem(a, g["a_f64"], 1e-2)
    assert rel_elem(mean, g["mean_f64"], 1e-2) < 1e-3, rel_elem(mean, g["mean_f64"], 1e-2)
    assert rel_elem(var, g["var_f64"]) < 1e-3, rel_elem(var, g["var_f64"])


@pytest.mark.gpu
def test_weight_and_precision_match_posterior(cuda_device):
    name = "ordinal_matern12_n200"
    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    gp = pg.LaplaceGP((g["X"], g["y"]), p.prior(), pg.log_probit_likelihood, tolerance=tol)
    a = gp.weight(p.params())
    W, f = gp.precision(a, p.params())
    assert rel_max(a, g["a_f64"]) < 1e-4
    assert rel_max(W, g["W_f64"]) < 1e-4
    assert rel_max(f, g["f_f64"]) < 1e-4
    # the fixed-point map at a* returns a* (f_LA(a*) = grad log p(K a*) = a*)
    fa = gp.construct()(p.params(), a)
    assert rel_max(fa, a) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("lik", ["gaussian", "probit", "probit_stable"])
def test_likelihood_kernel_matches_oracle(lik, cuda_device):
    """Per-point likelihood terms vs the float64 oracle.

    In the bulk (every class probability P >= 1e-2) all three forms match to
    float32 accuracy.  In the tails the reference form computes P as a
    difference of two float32 CDFs, which cancels to zero (log floor
    log 1e-10) exactly as the reference's float32 run does, and the stable
    form's d2 loses about eps * z^2 where the z^2 terms of its derivative
    cancel; there the checks are finiteness, the floor, and 1e-3 agreement.
    """
    from oracle import laplace as L

    rng = np.random.default_rng(5)
    cut = np.array([-np.inf, -1.0, 0.2, 1.1, np.inf])
    for lo, hi, bulk in ((-1.2, 1.2, True), (-8.0, 8.0, False)):
        f = rng.uniform(lo, hi, 2000).astype(np.float32)
        if lik == "gaussian":
            y = rng.normal(0, 1, 2000).astype(np.float32)
            lp, c, sig = (0.4,), None, 0.4
        else:
            y = rng.integers(0, 4, 2000).astype(np.int32)
            lp, c, sig = (0.7, cut), cut, 0.7
        ref = L.lik_terms(lik, f.astype(np.float64), y, sig, c, np.float64)
        got = LIK[lik](f, y, lp)
        assert np.isfinite(got).all()
        if lik == "gaussian" or bulk:
            mask = np.ones(f.size, bool)
            if lik != "gaussian":
                mask = np.exp(ref["logp"]) >= 1e-2
                assert mask.mean() > 0.5
            err = np.abs(got - ref["logp"])[mask]
            assert (err <= 2e-5 * np.maximum(1.0, np.abs(ref["logp"][mask]))).all(), err.max()
        elif lik == "probit":
            assert (got >= np.log(np.float32(1e-10)) - 1e-3).all()
        else:
            assert np.abs(got - ref["logp"]).max() <= 1e-3 * np.abs(ref["logp"]).max()
        if lik == "probit_stable":
            d1 = pg.grad_log_probit_likelihood(f, y, lp)
            d2 = pg.hessian_log_probit_likelihood(f, y, lp)
            assert np.isfinite(d1).all() and np.isfinite(d2).all()
            bar = 1e-4 if bulk else 1e-3
            assert np.abs(d1 - ref["d1"]).max() <= bar * np.abs(ref["d1"]).max()
            assert np.abs(d2 - ref["d2"]).max() <= bar * np.abs(ref["d2"]).max()


@pytest.mark.gpu
def test_gram_matches_oracle(native_lib, cuda_device):
    import torch
    from oracle import laplace as L

    rng = np.random.default_rng(7)
    for kind, code in (("eq", N.KERNEL_EQ), ("matern12", N.KERNEL_MATERN12), ("eq_periodic", N.KERNEL_EQ_PERIODIC)):
        X1 = rng.uniform(-2, 2, (150, 3)).astype(np.float32)
        X2 = rng.uniform(-2, 2, (70, 3)).astype(np.float32)
        ell = np.array([0.7, 1.1, 1.6])
        theta = torch.tensor(np.concatenate([ell, [1.3, 0.1]]), dtype=torch.float32, device="cuda")
        d = N.Desc(150, 3, code, 3, 0.5, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
        K = torch.zeros(150, 72, device="cuda")
        x1, x2 = torch.from_numpy(X1).cuda(), torch.from_numpy(X2).cuda()
        N.check(native_lib.pgb_gram(d, theta.data_ptr(), x1.data_ptr(), 150, x2.data_ptr(), 70, K.data_ptr(), 72,
                                    torch.cuda.current_stream().cuda_stream), "pgb_gram")
        ref = L.gram(kind, X1.astype(np.float64), X2.astype(np.float64), ell, 1.3, 0.5)
        # float32 sine of arguments up to ~25 rad: a few ulp of the argument
        assert np.abs(K[:, :70].cpu().numpy() - ref).max() < 1e-5, kind
        assert float(K[:, 70:].abs().max()) == 0.0


@pytest.mark.gpu
def test_not_positive_definite_gives_nan_and_status(cuda_device):
    """A negative signal variance makes B indefinite: NaN evidence, ENOTPD status."""
    name = "gauss_eq_ard_n400"
    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    gp = pg.LaplaceGP((g["X"], g["y"]), p.prior(), pg.log_gaussian_likelihood, tolerance=tol)
    ((ell, s), lik) = p.params()
    with pytest.warns(RuntimeWarning):
        v = gp.objective()(((ell, -4.0 * s), lik))
    assert np.isnan(v)
    code, _, col, _ = gp.last_status()
    assert code in (N.PGB_ENOTPD, N.PGB_ENAN) and col >= 0
    # the handle stays usable afterwards
    v2 = gp.objective()(p.params())
    assert abs(v2 - float(g["value_f64"])) <= 1e-4 * abs(float(g["value_f64"]))


@pytest.mark.gpu
def test_eager_mode_matches_graph_mode(cuda_device, monkeypatch):
    """PGB_EAGER=1 launches the same kernels without graphs: identical results."""
    name = "ordinal_matern12_n200"
    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    out = []
    for eager in ("0", "1"):
        monkeypatch.setenv("PGB_EAGER", eager)
        gp = pg.LaplaceGP((g["X"], g["y"]), p.prior(), pg.log_probit_likelihood, tolerance=tol)
        v, gr = gp.value_and_grad()(p.params())
        out.append((v, flat(gr), gp.last_status()[1]))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ordinal_matern12_n200", "ordinal_periodic_n130", "gauss_eq_ard_n400"])
def test_predict_covariance_and_distributions(name, cuda_device):
    """Full predictive covariance and ordinal predictive distributions against
    the oracle at the fitted posterior (bars: 1e-4 of s for covariance
    entries, 1e-4 absolute for probabilities)."""
    import ctypes as C

    import torch

    from oracle import laplace as L
    from cases import oracle_problem

    g = np.load(GOLD / f"{name}.npz")
    p, theta, tol = make(name)
    lik = CASES[name][1]
    gp = pg.LaplaceGP((g["X"], g["y"]), p.prior(), LIK[lik], tolerance=tol)
    params = p.params()
    a, W = gp.approximate_posterior(params)
    Xs = g["Xtest"]
    cov = gp.predict_covariance(Xs, params, a, W)
    mean, var = gp.predict(Xs, params, a, W)
    op = oracle_problem(p, lik)
    cov64 = L.predict_covariance(op, theta, Xs.astype(np.float64), np.asarray(a, np.float64),
                                 np.asarray(W, np.float64))
    s = p.variance
    assert cov.shape == (Xs.shape[0], Xs.shape[0])
    assert np.abs(cov - cov64).max() < 1e-4 * s, np.abs(cov - cov64).max()
    assert np.abs(np.diag(cov) - var).max() < 1e-5 * s
    assert np.allclose(cov, cov.T, atol=0)
    # the same with the factor rebuilt from W
    cov2 = gp.predict_covariance(Xs, params, np.array(a), np.array(W))
    assert np.abs(cov2 - cov).max() < 1e-5 * s
    if lik == "gaussian":
        return
    sigma, cut = params[1]
    d64 = L.predictive_distributions(sigma, cut, np.asarray(mean, np.float64), np.asarray(var, np.float64))
    dist = pg.probit_predictive_distributions(params[1], mean, var)
    assert dist.shape == d64.shape
    assert np.abs(dist - d64).max() < 1e-4
    assert np.allclose(dist.sum(axis=1), 1.0, atol=1e-5)
    # fused with predict through the C-ABI
    h = list(gp._handles.values())[0]
    dev = cuda_device
    M = Xs.shape[0]
    J = len(cut) - 1
    td = torch.tensor(theta, dtype=torch.float32, device=dev)
    Xd = torch.tensor(g["X"], dtype=torch.float32, device=dev)
    ad = torch.tensor(np.asarray(a), dtype=torch.float32, device=dev)
    Wd = torch.tensor(np.asarray(W), dtype=torch.float32, device=dev)
    Xsd = torch.tensor(Xs, dtype=torch.float32, device=dev)
    dd = torch.empty((M, J), dtype=torch.float32, device=dev)
    N.check(h.lib.pgb_predict_distributions(h.h, Xd.data_ptr(), td.data_ptr(), ad.data_ptr(), Wd.data_ptr(),
                                            Xsd.data_ptr(), M, dd.data_ptr(), None, None, 0,
                                            torch.cuda.current_stream().cuda_stream), "pgb_predict_distributions")
    torch.cuda.synchronize()
    assert np.abs(dd.cpu().numpy() - d64).max() < 1e-4
