"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference publishes no dataset; its examples draw latent functions from
the GP prior and threshold them (``examples/classification.py:181-322``,
``examples/regression.py:28-80``).  These generators do the same with NumPy
(float64 Cholesky of K + jitter I for the prior draw):

* ``ordinal_c0``: N=512, X ~ U[-2,2]^2, Matern12 (l=1, s=1), jitter 1e-6,
  y = bin(f + N(0, 0.4)) at cutpoints [-inf, -0.5, 0.5, inf], noise std
  sqrt(0.4) (the example's noise *variance* 0.4), predict on a 40 x 25 grid.
* ``regression_c1``: N=8192, X ~ N(0, I_4), EQ with ARD lengthscales
  (0.5, 1, 1.5, 2), s=1, noise std 0.2, predict at M=65,536 points ~ N(0, I_4).
* ``batched_c2`` / ``hyperopt_c3``: many ordinal problems with per-problem
  size, dimension, classes and kernel.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .kernels import EQ, Matern12


@dataclass
class Problem:
    """One synthetic GP problem and the hyperparameters it is fitted with."""

    X: np.ndarray
    y: np.ndarray
    kernel: str            # "eq" | "matern12" | "eq_periodic"
    lengthscale: np.ndarray
    variance: float
    noise_std: float
    cutpoints: np.ndarray | None = None   # J+1 with infinite ends (ordinal)
    period: float = 0.5
    Xtest: np.ndarray | None = None
    f: np.ndarray | None = None

    @property
    def N(self):
        return self.X.shape[0]

    @property
    def D(self):
        return self.X.shape[1]

    @property
    def J(self):
        return 0 if self.cutpoints is None else self.cutpoints.size - 1

    def prior(self):
        """``prior(params[0])`` callable in the reference's style."""
        kernel, period = self.kernel, self.period

        def prior(prior_parameters):
            ell, s = prior_parameters
            base = Matern12() if kernel == "matern12" else EQ()
            k = s * base.stretch(ell)
            return k.periodic(period) if kernel == "eq_periodic" else k

        return prior

    def params(self):
        ell = self.lengthscale if self.lengthscale.size > 1 else float(self.lengthscale[0])
        if self.cutpoints is None:
            return ((ell, self.variance), (self.noise_std,))
        return ((ell, self.variance), (self.noise_std, self.cutpoints))

    def theta(self):
        parts = [self.lengthscale.reshape(-1), [self.variance, self.noise_std]]
        if self.cutpoints is not None:
            parts.append(self.cutpoints)
        return np.concatenate(parts).astype(np.float64)


def gram64(kernel, X1, X2, ell, s, period=0.5):
    """Float64 kernel matrix for data generation."""
    ell = np.asarray(ell, dtype=np.float64).reshape(-1)
    X1 = np.asarray(X1, np.float64)
    X2 = np.asarray(X2, np.float64)
    if kernel == "eq_periodic":
        t = (X1[:, None, :] - X2[None, :, :]) * (math.pi / period)
        d2 = np.sum((2.0 * np.sin(t) / ell) ** 2, axis=2)
    else:
        d2 = np.zeros((X1.shape[0], X2.shape[0]))
        for d in range(X1.shape[1]):
            e = ell[0] if ell.size == 1 else ell[d]
            d2 += (X1[:, d:d + 1] / e - X2[None, :, d] / e) ** 2
    if kernel == "matern12":
        return s * np.exp(-np.sqrt(d2))
    return s * np.exp(-0.5 * d2)


def gram64_gemm(kernel, X, ell, s, period=0.5):
    """Float64 K(X, X) through matrix products, for large draws.

    Squared distances as |z_i|^2 + |z_j|^2 - 2 z_i.z_j with z = x / l, and for
    the periodic kernel sum_d (2 / l_d^2)(1 - cos(w x_id) cos(w x_jd)
    - sin(w x_id) sin(w x_jd)), w = 2 pi / period, which equals
    sum_d (2 sin(pi (x_id - x_jd) / period) / l_d)^2.
    """
    X = np.asarray(X, np.float64)
    D = X.shape[1]
    ell = np.broadcast_to(np.asarray(ell, dtype=np.float64).reshape(-1), (D,))
    if kernel == "eq_periodic":
        ang = X * (2.0 * math.pi / period)
        C, S = np.cos(ang), np.sin(ang)
        w = 2.0 / ell ** 2
        d2 = w.sum() - (C * w) @ C.T - (S * w) @ S.T
    else:
        Z = X / ell
        sq = np.einsum("ij,ij->i", Z, Z)
        d2 = sq[:, None] + sq[None, :] - 2.0 * (Z @ Z.T)
    np.maximum(d2, 0.0, out=d2)
    if kernel == "matern12":
        return s * np.exp(-np.sqrt(d2))
    return s * np.exp(-0.5 * d2)


def _draw_latent_torch(kernel, X, ell, s, period, jitter, z, device):
    """The large-draw path of draw_latent in float64 torch on `device`."""
    import torch

    Xt = torch.as_tensor(np.asarray(X, np.float64), device=device)
    D = Xt.shape[1]
    ell_t = torch.as_tensor(np.broadcast_to(np.asarray(ell, np.float64).reshape(-1), (D,)).copy(), device=device)
    if kernel == "eq_periodic":
        ang = Xt * (2.0 * math.pi / period)
        C, S = torch.cos(ang), torch.sin(ang)
        w = 2.0 / ell_t ** 2
        d2 = w.sum() - (C * w) @ C.T - (S * w) @ S.T
    else:
        Z = Xt / ell_t
        sq = (Z * Z).sum(1)
        d2 = sq[:, None] + sq[None, :] - 2.0 * (Z @ Z.T)
    d2.clamp_(min=0.0)
    K = s * (torch.exp(-torch.sqrt(d2)) if kernel == "matern12" else torch.exp(-0.5 * d2))
    K.diagonal().add_(jitter)
    L = torch.linalg.cholesky(K)
    return (L @ torch.as_tensor(z, device=device)).cpu().numpy()


def draw_latent(rng, kernel, X, ell, s, period=0.5, jitter=1e-6, device=None):
    """f ~ GP(0, K) at X (float64 Cholesky of K + jitter I).

    Draws of more than 1024 points build K by matrix products and factor it
    with SciPy's LAPACK Cholesky (or, given a torch `device`, in float64 on
    that device), which is much faster for large N; smaller draws keep the
    direct per-dimension form (the fixtures under tests/golden were generated
    with it).  The random numbers come from `rng` either way.
    """
    if X.shape[0] > 1024 and device is not None:
        z = rng.standard_normal(X.shape[0])
        try:
            return _draw_latent_torch(kernel, X, ell, s, period, jitter, z, device)
        except RuntimeError:
            # torch's linear-algebra library can be unavailable (e.g. under a
            # profiler that changes the library search path): same draw on the host
            import scipy.linalg as sla

            K = gram64_gemm(kernel, X, ell, s, period)
            K[np.diag_indices_from(K)] += jitter
            return sla.cholesky(K, lower=True, check_finite=False) @ z
    if X.shape[0] > 1024:
        import scipy.linalg as sla

        K = gram64_gemm(kernel, X, ell, s, period)
        K[np.diag_indices_from(K)] += jitter
        L = sla.cholesky(K, lower=True, check_finite=False)
    else:
        K = gram64(kernel, X, X, ell, s, period)
        K[np.diag_indices_from(K)] += jitter
        L = np.linalg.cholesky(K)
    return L @ rng.standard_normal(X.shape[0])


def ordinal_problem(rng, N, D, J, kernel, ell, s, noise_std, cut_interior, X_low=-2.0, X_high=2.0,
                    period=0.5, jitter=1e-6, n_test=0, device=None):
    X = rng.uniform(X_low, X_high, size=(N, D))
    ell = np.atleast_1d(np.asarray(ell, dtype=np.float64))
    f = draw_latent(rng, kernel, X, ell, s, period, jitter, device)
    g = f + noise_std * rng.standard_normal(N)
    cut = np.concatenate([[-np.inf], np.asarray(cut_interior, dtype=np.float64), [np.inf]])
    y = np.searchsorted(cut[1:-1], g).astype(np.int32)
    Xt = rng.uniform(X_low, X_high, size=(n_test, D)).astype(np.float32) if n_test else None
    return Problem(X.astype(np.float32), y, kernel, ell, float(s), float(noise_std), cut, period, Xt,
                   f.astype(np.float32))


def regression_problem(rng, N, D, kernel, ell, s, noise_std, period=0.5, jitter=1e-6, n_test=0, device=None):
    X = rng.standard_normal((N, D))
    ell = np.atleast_1d(np.asarray(ell, dtype=np.float64))
    f = draw_latent(rng, kernel, X, ell, s, period, jitter, device)
    y = f + noise_std * rng.standard_normal(N)
    Xt = rng.standard_normal((n_test, D)).astype(np.float32) if n_test else None
    return Problem(X.astype(np.float32), y.astype(np.float32), kernel, ell, float(s), float(noise_std), None,
                   period, Xt, f.astype(np.float32))


def ordinal_c0() -> Problem:
    rng = np.random.default_rng(0)
    p = ordinal_problem(rng, 512, 2, 3, "matern12", 1.0, 1.0, math.sqrt(0.4), [-0.5, 0.5])
    gx, gy = np.meshgrid(np.linspace(-2, 2, 40), np.linspace(-2, 2, 25), indexing="ij")
    p.Xtest = np.stack([gx.ravel(), gy.ravel()], axis=1).astype(np.float32)
    return p


def regression_c1(N=8192, M=65536, device=None) -> Problem:
    rng = np.random.default_rng(1)
    return regression_problem(rng, N, 4, "eq", [0.5, 1.0, 1.5, 2.0], 1.0, 0.2, n_test=M, device=device)


def _cut_interior(J):
    return [0.0] if J == 2 else list(np.linspace(-1.5, 1.5, J - 1))


def batched_c2(B=1024, n_min=32, n_max=4096, seed=2, device=None) -> list[Problem]:
    rng = np.random.default_rng(seed)
    kinds = ["eq", "matern12", "eq_periodic"]
    out = []
    for _ in range(B):
        N = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        D = int(rng.choice([1, 2, 4, 8]))
        J = int(rng.integers(2, 8))
        kind = kinds[int(rng.integers(0, 3))]
        ell = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
        s = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        out.append(ordinal_problem(rng, N, D, J, kind, ell, s, math.sqrt(0.4), _cut_interior(J), device=device))
    return out


def hyperopt_c3(B=256, seed=3, device=None) -> list[Problem]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(B):
        N = int(rng.integers(256, 2049))
        out.append(ordinal_problem(rng, N, 3, 5, "matern12", 1.0, 1.0, math.sqrt(0.4), _cut_interior(5),
                                   device=device))
    return out


def serving_c4(rate=2000.0, duration=60.0, pool=256, seed=4, n_min=32, n_max=8192, device=None):
    """The serving workload: a pool of `pool` ordinal GPs generated as in
    ``batched_c2`` (N log-uniform in [n_min, n_max], D in 1..8, J in 2..7,
    kernel in {EQ, Matern12, EQ.periodic(0.5)}) and Poisson arrivals at
    `rate` requests/s for `duration` s: 70% predict (M log-uniform in
    [1, 4096] test points ~ U[-2, 2]^D against a fitted model of the pool),
    20% fit (refit of a pool model), 10% evidence + gradient (a pool model's
    data at hyperparameters scaled by U[0.8, 1.25]).

    Returns (problems, requests) with serving.Problem / serving.Request
    objects; the caller fits every pool model before replaying the requests.
    """
    from . import serving as S

    rng = np.random.default_rng(seed)
    kinds = ["eq", "matern12", "eq_periodic"]
    problems = []
    for _ in range(pool):
        N = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        D = int(rng.integers(1, 9))
        J = int(rng.integers(2, 8))
        kind = kinds[int(rng.integers(0, 3))]
        ell = math.exp(rng.uniform(math.log(0.3), math.log(3.0)))
        s = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        p = ordinal_problem(rng, N, D, J, kind, ell, s, math.sqrt(0.4), _cut_interior(J), device=device)
        problems.append(S.Problem(p.X, p.y, kind, p.theta().astype(np.float32), 1, J, p.period))
    requests = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        u = rng.uniform()
        k = int(rng.integers(0, pool))
        p = problems[k]
        if u < 0.7:
            M = int(round(math.exp(rng.uniform(0.0, math.log(4096)))))
            Xs = rng.uniform(-2.0, 2.0, size=(M, p.d)).astype(np.float32)
            requests.append(S.Request(t, "predict", k, p, Xs=Xs))
        elif u < 0.9:
            requests.append(S.Request(t, "fit", k, p))
        else:
            th = p.theta.copy()
            th[:3] *= rng.uniform(0.8, 1.25, size=3).astype(np.float32)
            requests.append(S.Request(t, "vg", k, p, theta=th))
    return problems, requests
