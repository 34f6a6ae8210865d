"""The near band autotuner and whole-problem blocks on the GPU: results agree
across near band depths, the tuner times real evaluations, and problems of
at most two tile rows factored whole by one block give the bits of the
tile-per-task order.  Files named test_zz_* are collected after the core
parity suite."""

import numpy as np
import pytest

from probit_gb300 import autotune as A


@pytest.mark.gpu
def test_depths_agree_and_tuner_runs(cuda_device):
    import probit_gb300 as pg
    from probit_gb300 import workloads as W

    p = W.regression_problem(np.random.default_rng(3), 1000, 3, "eq", np.array([0.6, 1.0, 1.4]), 1.0, 0.3)
    vals = {}
    for q in (1, 2, 5):
        A.use(A.Table("t", [A.Entry(1, 1 << 20, q, 1000, {q: 1.0})]))
        try:
            gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_gaussian_likelihood, tolerance=1e-3)
            v, g = gp.value_and_grad()(p.params())
            vals[q] = (float(v), np.concatenate([np.ravel(np.asarray(x, np.float64)) for x in
                                                 [g[0][0], g[0][1], g[1][0]]]))
        finally:
            A.use(None)
    for q in (2, 5):
        assert abs(vals[q][0] - vals[1][0]) <= 1e-5 * abs(vals[1][0])
        assert np.allclose(vals[q][1], vals[1][1], rtol=1e-3, atol=1e-4)
    t = A.tune(A.gpu_timer(reps=2, warmup=1), buckets=((1, 2), (5, 8)), candidates=(1, 2, 3))
    assert [e.depth for e in t.entries] and all(1 <= e.depth <= 3 for e in t.entries)
    assert all(ms > 0 for e in t.entries for ms in e.ms.values())


@pytest.mark.gpu
@pytest.mark.parametrize("n", [90, 200, 256])
def test_whole_problem_blocks_give_the_same_bits(cuda_device, monkeypatch, n):
    """A problem of at most two tile rows factored whole by one block gives
    the bits of the tile-per-task order (same tile arithmetic, same order)."""
    import probit_gb300 as pg
    from probit_gb300 import workloads as W

    p = W.ordinal_problem(np.random.default_rng(n), n, 2, 3, "matern12", 0.9, 1.1, 0.6, [-0.5, 0.5])
    out = {}
    for whole in ("0", "2"):
        monkeypatch.setenv("PGB_WHOLE_TILES", whole)
        gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=1e-4)
        v, g = gp.value_and_grad()(p.params())
        a, W_ = gp.approximate_posterior(p.params())
        out[whole] = (np.float32(v), np.asarray(a), np.asarray(W_), np.asarray(g[0][0]), np.asarray(g[1][1]))
    # bitwise, each output in its own dtype (the isotropic lengthscale's
    # gradient comes back as a 0-d float64)
    for x, y in zip(out["0"], out["2"]):
        x, y = np.asarray(x), np.asarray(y)
        assert x.dtype == y.dtype and x.shape == y.shape
        assert x.tobytes() == y.tobytes()
