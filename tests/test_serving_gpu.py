"""Serving (probit_gb300.serving): requests in a concurrent mix give what
they give alone, and predicts reuse the resident factor of their model."""

import numpy as np
import pytest

from probit_gb300 import serving as S
from probit_gb300 import workloads as W


@pytest.fixture(scope="module")
def trace(cuda_device):
    problems, requests = W.serving_c4(rate=400.0, duration=0.25, pool=8, n_max=700, seed=41)
    return problems, requests


def _fits(problems):
    return [S.Request(0.0, "fit", k, p) for k, p in enumerate(problems)]


def _run(problems, requests, workers, sequential, **server_kw):
    srv = S.Server(workers=workers, mem_budget=8 << 30, **server_kw)
    try:
        srv.replay(_fits(problems), realtime=False)
        if sequential:
            out = []
            for r in requests:
                srv.replay([r], realtime=False)
                out.append(r)
            return out
        return srv.replay(requests, realtime=False)
    finally:
        srv.close()


def _clone(reqs):
    return [S.Request(r.arrival, r.kind, r.model, r.problem, Xs=r.Xs, theta=r.theta) for r in reqs]


@pytest.mark.gpu
def test_same_alone_and_in_the_mix(trace):
    problems, requests = trace
    assert len(requests) >= 40
    alone = _run(problems, _clone(requests), workers=1, sequential=True)
    mixed = _run(problems, _clone(requests), workers=8, sequential=False)
    kinds = set()
    for a, m in zip(alone, mixed):
        assert a.error is None and m.error is None, (a.error, m.error)
        kinds.add(a.kind)
        for x, y in zip(a.result, m.result):
            assert np.array_equal(np.asarray(x), np.asarray(y)), (a.kind, a.model)
    assert kinds == {"fit", "vg", "predict"}


@pytest.mark.gpu
def test_block_caps_keep_results(trace):
    """Capping a model's launches to a few blocks (the persistent ones, and
    the matvec / gradient-trace grids, whose blocks then stride over their
    maps) changes no bit of any result."""
    problems, requests = trace
    free = _run(problems, _clone(requests), workers=4, sequential=False)
    capped = _run(problems, _clone(requests), workers=4, sequential=False, small_n=300, large_blocks=2,
                  small_blocks=3, max_large=2)
    assert any(p.n > 300 for p in problems) and any(p.n <= 300 for p in problems)
    for a, m in zip(free, capped):
        assert a.error is None and m.error is None, (a.error, m.error)
        for x, y in zip(a.result, m.result):
            assert np.array_equal(np.asarray(x), np.asarray(y)), (a.kind, a.model)


@pytest.mark.gpu
def test_predict_matches_laplacegp(trace):
    """A served predict equals LaplaceGP.predict on the same model."""
    import probit_gb300 as pg

    problems, requests = trace
    k = 3
    p = problems[k]
    srv = S.Server(workers=2, mem_budget=4 << 30)
    try:
        srv.replay([S.Request(0.0, "fit", k, p)], realtime=False)
        Xs = np.random.default_rng(5).uniform(-2, 2, size=(300, p.d)).astype(np.float32)
        r = srv.replay([S.Request(0.0, "predict", k, p, Xs=Xs)], realtime=False)[0]
    finally:
        srv.close()
    assert r.error is None
    cut = p.theta[3:]

    def prior(pp):
        ell, s = pp
        k_ = s * (pg.Matern12() if p.kind == "matern12" else pg.EQ()).stretch(ell)
        return k_.periodic(p.period) if p.kind == "eq_periodic" else k_

    gp = pg.LaplaceGP((p.X, p.y), prior, pg.log_probit_likelihood, tolerance=p.tolerance)
    params = ((float(p.theta[0]), float(p.theta[1])), (float(p.theta[2]), cut.astype(np.float64)))
    a, W_ = gp.approximate_posterior(params)
    mean, var = gp.predict(Xs, params, a, W_)
    assert np.abs(r.result[0] - mean).max() <= 1e-5 * max(1.0, np.abs(mean).max())
    assert np.abs(r.result[1] - var).max() <= 1e-5


@pytest.mark.gpu
def test_admission_by_memory(trace):
    """With a budget for about two models, requests still all complete, idle
    models are evicted, and the accounted HBM never exceeds the budget."""
    problems, requests = trace
    big = max(S.handle_bytes(p.n, p.d, p.kind, grad=True, m=4096) for p in problems)
    srv = S.Server(workers=4, mem_budget=int(1.5 * big))
    peak = [0]
    try:
        srv.replay(_fits(problems), realtime=False)
        reqs = _clone([r for r in requests if r.kind != "predict"])
        for r in reqs:
            srv.submit(r)
        import time
        while any(r.done is None for r in reqs):
            peak[0] = max(peak[0], srv.used)
            time.sleep(0.001)
    finally:
        srv.close()
    assert all(r.error is None for r in reqs)
    assert peak[0] <= srv.budget
    assert srv.evictions > 0
