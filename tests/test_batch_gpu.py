"""Batched evaluation (pgb_batch_*) through the C-ABI.

A batch of problems of different sizes (N not a multiple of the 128-row
tile, one tile, several tiles), input dimensions, kernel families, class
counts and likelihoods must give, for every problem, what the single-GP path
gives for that problem alone, and agree with the float64 oracle to the
parity bars (negative log evidence 1e-4 relative, gradient 1e-3 of its
largest entry, Newton iterations within 1 of the float32 oracle).
"""

import math

import numpy as np
import pytest

import probit_gb300 as pg
from probit_gb300 import workloads as W

# (N, D, J, kernel); J = 0 is Gaussian regression
SPECS = [(40, 1, 2, "eq"), (128, 2, 3, "matern12"), (129, 4, 5, "eq_periodic"), (200, 8, 7, "eq"),
         (300, 2, 4, "matern12"), (513, 1, 2, "eq_periodic"), (90, 4, 3, "matern12"), (256, 3, 0, "eq"),
         (700, 2, 3, "eq"), (1, 2, 3, "matern12")]


def _problems(seed=21):
    rng = np.random.default_rng(seed)
    out = []
    for N, D, J, kind in SPECS:
        ell = float(np.exp(rng.uniform(np.log(0.5), np.log(2.0))))
        s = float(np.exp(rng.uniform(np.log(0.6), np.log(1.6))))
        if J == 0:
            p = W.regression_problem(rng, N, D, kind, ell, s, 0.3)
        else:
            interior = [0.0] if J == 2 else list(np.linspace(-1.2, 1.2, J - 1))
            p = W.ordinal_problem(rng, N, D, J, kind, ell, s, math.sqrt(0.4), interior)
        out.append(p)
    return out


def _tol(p):
    return 1e-3 if p.cutpoints is None else 1e-4


def _gp(p):
    lik = pg.log_gaussian_likelihood if p.cutpoints is None else pg.log_probit_likelihood
    return pg.LaplaceGP((p.X, p.y), p.prior(), lik, tolerance=_tol(p))


def _flat(tree):
    from probit_gb300.approximators import tree_leaves

    return np.concatenate([np.atleast_1d(np.asarray(v, np.float64)) for v in tree_leaves(tree)])


@pytest.fixture(scope="module")
def batch_run(cuda_device):
    probs = _problems()
    gps = [_gp(p) for p in probs]
    params = [p.params() for p in probs]
    batch = pg.LaplaceBatch(gps, params)
    values, grads = batch.value_and_grad()(params)
    return probs, gps, params, batch, values, grads


@pytest.mark.gpu
def test_batch_matches_single_path(batch_run):
    probs, gps, params, batch, values, grads = batch_run
    st = batch.status()
    for b, (p, gp) in enumerate(zip(probs, gps)):
        v1, g1 = gp.value_and_grad()(params[b])
        it1 = gp.last_status()[1]
        assert st[b][0] == 0, (b, st[b])
        assert st[b][1] == it1, (b, st[b][1], it1)
        assert abs(values[b] - v1) <= 1e-6 * max(1.0, abs(v1)), (b, values[b], v1)
        gb, gs = _flat(grads[b]), _flat(g1)
        assert np.abs(gb - gs).max() <= 1e-5 * max(np.abs(gs).max(), 1e-30), (b, gb, gs)


@pytest.mark.gpu
def test_batch_matches_oracle(batch_run):
    from oracle import laplace as L

    probs, gps, params, batch, values, grads = batch_run
    st = batch.status()
    for b, p in enumerate(probs):
        lik = "gaussian" if p.cutpoints is None else "probit"
        op = L.Problem(p.X.astype(np.float64), p.y, p.kernel, lik, p.lengthscale.size, p.period, p.J)
        v64, g64, _, _ = L.value_and_grad(op, p.theta(), tol=_tol(p), dtype=np.float64)
        _, _, _, it32 = L.value_and_grad(op, p.theta(), tol=_tol(p), dtype=np.float32)
        assert abs(values[b] - v64) <= 1e-4 * abs(v64), (b, values[b], v64)
        gb = _flat(grads[b])
        assert np.abs(gb - g64).max() <= 1e-3 * np.abs(g64).max(), (b, gb, g64)
        assert abs(st[b][1] - it32) <= 1, (b, st[b][1], it32)


@pytest.mark.gpu
def test_batch_objective_and_repeat(batch_run):
    """objective() gives the values of value_and_grad(); a second call (graph replay) the same bits."""
    probs, gps, params, batch, values, grads = batch_run
    v = batch.objective()(params)
    assert np.allclose(v, values, rtol=1e-6, atol=0)
    values2, grads2 = batch.value_and_grad()(params)
    assert np.array_equal(values2, values)
    for g1, g2 in zip(grads, grads2):
        assert np.array_equal(_flat(g1), _flat(g2))


@pytest.mark.gpu
def test_batch_result_independent_of_company(batch_run):
    """A problem gives the same result alone, in this batch, and in a batch ordered differently."""
    probs, gps, params, batch, values, grads = batch_run
    order = [9, 3, 8, 0, 5, 1, 7, 2, 6, 4]
    b2 = pg.LaplaceBatch([gps[k] for k in order], [params[k] for k in order])
    v2, g2 = b2.value_and_grad()([params[k] for k in order])
    for pos, k in enumerate(order):
        assert abs(v2[pos] - values[k]) <= 1e-6 * max(1.0, abs(values[k])), (k, v2[pos], values[k])
        assert np.allclose(_flat(g2[pos]), _flat(grads[k]), rtol=1e-5, atol=1e-6 * np.abs(_flat(grads[k])).max())


@pytest.mark.gpu
def test_batch_mask_evaluates_only_enabled(batch_run):
    """Disabled problems keep their last outputs; enabled ones equal a full evaluation."""
    import torch

    probs, gps, params, batch, values, grads = batch_run
    _, th1 = batch.pack_theta(params)
    th2 = th1.clone()
    off = batch.theta_off
    for b in range(batch.B):      # scale every signal variance by 1.1
        th2[int(off[b]) + int(batch.descs[b].n_lengthscales)] *= 1.1
    batch.set_enabled(None)
    v1, g1 = (t.clone() for t in batch.value_and_grad_flat(th1))
    v2, g2 = (t.clone() for t in batch.value_and_grad_flat(th2))
    mask = np.arange(batch.B) % 2 == 0
    batch.value_and_grad_flat(th1)                       # back to theta1 everywhere
    batch.set_enabled(mask)
    vm, gm = (t.clone() for t in batch.value_and_grad_flat(th2))
    batch.set_enabled(None)
    for b in range(batch.B):
        sl = slice(int(off[b]), int(off[b + 1]))
        if mask[b]:
            assert torch.equal(vm[b], v2[b]) and torch.equal(gm[sl], g2[sl]), b
        else:
            assert torch.equal(vm[b], v1[b]) and torch.equal(gm[sl], g1[sl]), b
