"""NumPy/SciPy restatement of the reference Laplace path (TEST INFRASTRUCTURE).

Every function names the reference file:line (paths inside bb515/probit) whose
arithmetic it restates.  Arrays are computed in the dtype passed in
(``np.float32`` mirrors the reference's float32 JAX run, ``np.float64`` its
``JAX_ENABLE_X64=1`` run).  Parity status: unpinned (see ``oracle/__init__``).

Hyperparameter vector layout used throughout (the same layout the CUDA
library's C-ABI uses): ``theta = [l_0 .. l_{nl-1}, s, sigma_n, b_0 .. b_J]``
with ``nl`` = 1 (isotropic) or D (ARD), ``s`` the signal variance, ``sigma_n``
the likelihood noise std and ``b`` the J+1 ordinal cutpoints (probit only,
``b_0 = -inf``, ``b_J = +inf``).
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
from scipy import linalg as sla
from scipy.special import erf, log_ndtr

__all__ = [
    "KERNELS", "LIKELIHOODS", "Problem", "h", "ndtr", "norm_cdf",
    "scaled_sq_dists", "gram", "gram_diag", "lik_terms", "newton_weight",
    "precision", "objective", "value_and_grad", "predict", "predict_covariance",
    "predictive_distributions", "objective_bform", "newton_weight_bform",
    "vb_map", "vb_weight", "vb_objective", "vb_objective_bform", "vb_value_and_grad",
]

KERNELS = ("eq", "matern12", "eq_periodic")
LIKELIHOODS = ("gaussian", "probit", "probit_stable")

SQRT2 = math.sqrt(2.0)
LOG_OVER_SQRT_2PI = -0.5 * math.log(2.0 * math.pi)   # utilities.py:11
OVER_SQRT_2PI = 1.0 / math.sqrt(2.0 * math.pi)       # utilities.py:10
PROBIT_EPS = 1e-10                                     # utilities.py:57


@dataclass
class Problem:
    """One GP problem: data, kernel family and likelihood family."""

    X: np.ndarray            # (N, D)
    y: np.ndarray            # (N,) float (gaussian) or int classes (probit)
    kernel: str = "eq"       # one of KERNELS
    likelihood: str = "gaussian"
    n_lengthscales: int = 1  # 1 or D
    period: float = 0.5      # EQ.periodic(period)
    J: int = 0               # ordinal classes (probit)
    distance: str = "diff"   # "diff" or "expanded"

    @property
    def N(self):
        return self.X.shape[0]

    @property
    def D(self):
        return self.X.shape[1]

    def split(self, theta):
        theta = np.asarray(theta)
        nl = self.n_lengthscales
        ell = theta[:nl]
        s = theta[nl]
        sig = theta[nl + 1]
        cut = theta[nl + 2:nl + 3 + self.J] if self.likelihood != "gaussian" else None
        return ell, s, sig, cut

    @property
    def n_theta(self):
        return self.n_lengthscales + 2 + (self.J + 1 if self.likelihood != "gaussian" else 0)


# ---------------------------------------------------------------- utilities

def h(x):
    """Tail-series polynomial; restates ``utilities.py:37-44``."""
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return -1 * x ** -2 + 5 / 2 * x ** -4 - 37 / 3 * x ** -6


def ndtr(z):
    """Phi(z) = 0.5 (1 + erf(z / sqrt 2)); restates ``utilities.py:18-19``."""
    z = np.asarray(z)
    dt = z.dtype.type
    return dt(0.5) * (dt(1) + erf(z / dt(SQRT2)).astype(z.dtype))


def norm_cdf(x):
    """Phi with +-inf guards; restates ``utilities.py:31-34``."""
    x = np.asarray(x)
    safe = np.where(np.isinf(x), x.dtype.type(1), x)
    extrema = np.where(x == np.inf, x.dtype.type(1), x.dtype.type(0))
    return np.where(np.isinf(x), extrema, ndtr(safe))


# ---------------------------------------------------------------- kernels

def _features(kernel, X, ell, period, dtype):
    """Inputs after ``.stretch`` (and ``.periodic``) as mlkernels composes them."""
    X = np.asarray(X, dtype=dtype)
    ell = np.asarray(ell, dtype=dtype).reshape(-1)
    if kernel == "eq_periodic":
        ang = X * dtype(2 * math.pi / period)
        sin, cos = np.sin(ang), np.cos(ang)
        return np.concatenate([sin / ell, cos / ell], axis=1)
    return X / ell


def scaled_sq_dists(kernel, X1, X2, ell, period=0.5, dtype=np.float64):
    """Per-dimension scaled squared distances q[i, j, d].

    ``eq``/``matern12``: q_d = (x_d/l_d - z_d/l_d)^2 (stretch divides the
    inputs first, as mlkernels' ``stretch`` does).  ``eq_periodic``:
    q_d = (2 sin(pi (x_d - z_d) / p) / l_d)^2, which equals the squared
    distance of the (sin, cos) features of ``EQ().stretch(l).periodic(p)``.
    """
    X1 = np.asarray(X1, dtype=dtype)
    X2 = np.asarray(X2, dtype=dtype)
    ell = np.asarray(ell, dtype=dtype).reshape(-1)
    if kernel == "eq_periodic":
        t = (X1[:, None, :] - X2[None, :, :]) * dtype(math.pi / period)
        v = dtype(2) * np.sin(t) / ell
        return v * v
    U1 = X1 / ell
    U2 = X2 / ell
    d = U1[:, None, :] - U2[None, :, :]
    return d * d


def gram(kernel, X1, X2, ell, s, period=0.5, dtype=np.float64, distance="diff"):
    """``B.dense(prior(theta)(X1, X2))``: s * k(r) for the supported family.

    Restates the kernel algebra that ``Laplace.py:7,21,24`` and
    ``approximators.py:172-174,272`` reach through mlkernels/lab.
    """
    dt = np.dtype(dtype).type
    if distance == "expanded":
        F1 = _features(kernel, X1, ell, period, dt)
        F2 = _features(kernel, X2, ell, period, dt)
        if F1.shape[1] == 1:
            d = F1 - F2.T
            d2 = d * d
            r = np.abs(d)
        else:
            n1 = np.sum(F1 * F1, axis=1)[:, None]
            n2 = np.sum(F2 * F2, axis=1)[None, :]
            d2 = np.maximum(n1 + n2 - dt(2) * (F1 @ F2.T), dt(0))
            r = np.sqrt(np.maximum(d2, dt(1e-12)))
    else:
        q = scaled_sq_dists(kernel, X1, X2, ell, period, dt)
        d2 = np.sum(q, axis=2, dtype=dt)
        r = np.sqrt(d2)
    if kernel == "matern12":
        k = np.exp(-r)
    else:
        k = np.exp(dt(-0.5) * d2)
    return (dt(s) * k).astype(dt)


def gram_diag(kernel, X, s, dtype=np.float64):
    """``kernel.elwise(X, X)`` for a stationary kernel: s * k(0) = s."""
    return np.full(np.asarray(X).shape[0], s, dtype=dtype)


def gram_param_derivs(kernel, X, ell, s, period=0.5, rows=None):
    """dK/dtheta_k for theta_k in (l_0..l_{nl-1}, s), float64, rows subset.

    Returns (K_rows, [dK/dl_0, ..., dK/ds]) each of shape (len(rows), N).
    """
    X = np.asarray(X, dtype=np.float64)
    ell = np.asarray(ell, dtype=np.float64).reshape(-1)
    rows = slice(None) if rows is None else rows
    q = scaled_sq_dists(kernel, X[rows], X, ell, period, np.float64)
    d2 = q.sum(axis=2)
    if kernel == "matern12":
        r = np.sqrt(d2)
        K = s * np.exp(-r)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv_r = np.where(r > 0, 1.0 / r, 0.0)
        scale = K * inv_r
    else:
        K = s * np.exp(-0.5 * d2)
        scale = K
    out = []
    if ell.size == 1:
        out.append(scale * d2 / ell[0])
    else:
        for d in range(ell.size):
            out.append(scale * q[:, :, d] / ell[d])
    out.append(K / s)
    return K, out


# ---------------------------------------------------------------- likelihoods

def _log_phi(z):
    return LOG_OVER_SQRT_2PI - 0.5 * z * z


def lik_terms(likelihood, f, y, sigma, cutpoints=None, dtype=np.float64):
    """Per-point log p, its f-derivatives d1..d3 and theta_lik partials.

    * ``gaussian``: ``log_gaussian_likelihood`` (``utilities.py:60-61,64-70``).
    * ``probit``: ``log_probit_likelihood`` = log(Z + 1e-10) with
      Z = Phi((b_{y+1}-f)/s) - Phi((b_y-f)/s) through erf and the +-inf guards
      (``utilities.py:47-57,195-229``); its derivatives are what JAX autodiff
      of that expression gives (``approximators.py:92-95``).
    * ``probit_stable``: the same model with log Z evaluated in log space
      (log_ndtr / erfcx form), no +1e-10.

    Derivatives of G(z1, z2) = log P are built from G_1 = -phi(z1)/P and
    G_2 = phi(z2)/P: G_11 = -z1 G_1 - G_1^2, G_22 = -z2 G_2 - G_2^2,
    G_12 = -G_1 G_2 and their next derivatives, then mapped to f, sigma and
    the two cutpoints through z_k = (b_k - f)/sigma.
    """
    dt = np.dtype(dtype).type
    f = np.asarray(f, dtype=dt)
    sig = dt(sigma)
    out = {}
    if likelihood == "gaussian":
        yv = np.asarray(y, dtype=dt)
        z = (f - yv) / sig
        out["logp"] = dt(LOG_OVER_SQRT_2PI) - z * z / dt(2) - np.log(sig)
        out["d1"] = (yv - f) / (sig * sig)
        out["d2"] = np.full_like(f, -dt(1) / (sig * sig))
        out["d3"] = np.zeros_like(f)
        out["dlogp_dsig"] = (z * z - dt(1)) / sig
        out["dd1_dsig"] = dt(-2) * (yv - f) / (sig * sig * sig)
        out["dd2_dsig"] = np.full_like(f, dt(2) / (sig * sig * sig))
        return out

    yi = np.asarray(y).astype(np.int64)
    cut = np.asarray(cutpoints, dtype=dt)
    b_lo = cut[yi]
    b_hi = cut[yi + 1]
    fin1 = np.isfinite(b_lo)
    fin2 = np.isfinite(b_hi)
    with np.errstate(all="ignore"):
        z1 = np.where(fin1, (np.where(fin1, b_lo, dt(0)) - f) / sig, dt(0))
        z2 = np.where(fin2, (np.where(fin2, b_hi, dt(0)) - f) / sig, dt(0))
        if likelihood == "probit":
            phi1 = np.where(fin1, ndtr(z1), dt(0))
            phi2 = np.where(fin2, ndtr(z2), dt(1))
            Pe = (phi2 - phi1) + dt(PROBIT_EPS)
            logp = np.log(Pe)
            pdf1 = dt(OVER_SQRT_2PI) * np.exp(dt(-0.5) * z1 * z1)
            pdf2 = dt(OVER_SQRT_2PI) * np.exp(dt(-0.5) * z2 * z2)
            G1 = np.where(fin1, -pdf1 / Pe, dt(0))
            G2 = np.where(fin2, pdf2 / Pe, dt(0))
        elif likelihood == "probit_stable":
            z1d = z1.astype(np.float64)
            z2d = z2.astype(np.float64)
            lo = np.where(fin1, log_ndtr(z1d), -np.inf)          # log Phi(z1)
            hi = np.where(fin2, log_ndtr(z2d), 0.0)              # log Phi(z2)
            q1 = np.where(fin1, log_ndtr(-z1d), 0.0)             # log Q(z1)
            q2 = np.where(fin2, log_ndtr(-z2d), -np.inf)         # log Q(z2)
            upper = fin1 & (z1d >= 0)
            lower = fin2 & (z2d <= 0) & ~upper
            mid = ~(upper | lower)
            logP = np.empty_like(z1d)
            logP[upper] = q1[upper] + np.log1p(-np.exp(q2[upper] - q1[upper]))
            logP[lower] = hi[lower] + np.log1p(-np.exp(lo[lower] - hi[lower]))
            logP[mid] = np.log1p(-(np.exp(lo[mid]) + np.exp(q2[mid])))
            logp = logP.astype(dt)
            G1 = np.where(fin1, -np.exp(_log_phi(z1d) - logP), 0.0).astype(dt)
            G2 = np.where(fin2, np.exp(_log_phi(z2d) - logP), 0.0).astype(dt)
        else:
            raise ValueError(likelihood)

        G11 = -z1 * G1 - G1 * G1
        G22 = -z2 * G2 - G2 * G2
        G12 = -G1 * G2
        G111 = -G1 - z1 * G11 - dt(2) * G1 * G11
        G112 = -z1 * G12 - dt(2) * G1 * G12
        G122 = -z2 * G12 - dt(2) * G2 * G12
        G222 = -G2 - z2 * G22 - dt(2) * G2 * G22
        isg = dt(1) / sig
        S2 = G11 + dt(2) * G12 + G22
        dS2_1 = G111 + dt(2) * G112 + G122
        dS2_2 = G112 + dt(2) * G122 + G222
        out["logp"] = logp
        out["d1"] = -(G1 + G2) * isg
        out["d2"] = S2 * isg * isg
        out["d3"] = -(G111 + dt(3) * G112 + dt(3) * G122 + G222) * isg ** 3
        out["dlogp_dsig"] = -(z1 * G1 + z2 * G2) * isg
        out["dd1_dsig"] = (z1 * (G11 + G12) + z2 * (G12 + G22) + G1 + G2) * isg * isg
        out["dd2_dsig"] = -(z1 * dS2_1 + z2 * dS2_2 + dt(2) * S2) * isg ** 3
        out["dlogp_dlo"] = G1 * isg
        out["dd1_dlo"] = -(G11 + G12) * isg * isg
        out["dd2_dlo"] = dS2_1 * isg ** 3
        out["dlogp_dhi"] = G2 * isg
        out["dd1_dhi"] = -(G12 + G22) * isg * isg
        out["dd2_dhi"] = dS2_2 * isg ** 3
        out["y"] = yi
    return out


# ---------------------------------------------------------------- Newton

def _K(prob: Problem, theta, dtype):
    ell, s, _, _ = prob.split(theta)
    return gram(prob.kernel, prob.X, prob.X, ell, s, prob.period, dtype, prob.distance)


def newton_weight(prob: Problem, theta, tol=1e-5, maxiter=100, dtype=np.float64, K=None):
    """``LaplaceGP.weight`` (``approximators.py:265-269``).

    ``newton_solver`` (``solvers.py:18-25``) with the jaxopt
    ``FixedPointIteration`` loop of ``fwd_solver`` (``solvers.py:7-15``):
    z <- z - J^-1 (F(z) - z), J = diag(d2) K - I built densely and solved by
    LU, from z_0 = 0; at most ``maxiter`` updates, stop once
    ||z_k - z_{k-1}||_2 <= tol (a NaN error also stops, as ``err > tol`` is
    false).  Returns (a, iterations).
    """
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    N = K.shape[0]
    z = np.zeros(N, dtype=dt)
    eye = np.eye(N, dtype=dt)
    it = 0
    while True:
        f = K @ z
        t = lik_terms(prob.likelihood, f, prob.y, sig, cut, dt)
        J = t["d2"][:, None] * K - eye
        r = t["d1"] - z
        with np.errstate(all="ignore"):
            try:
                step = sla.solve(J, r, check_finite=False)
            except (sla.LinAlgError, ValueError):
                step = np.full(N, np.nan, dtype=dt)
        z_new = (z - step.astype(dt)).astype(dt)
        err = np.sqrt(np.sum((z_new - z) ** 2, dtype=dt))
        z = z_new
        it += 1
        if not (err > tol) or it >= maxiter:
            break
    return z, it


def precision(prob: Problem, theta, a, dtype=np.float64, K=None):
    """``LaplaceGP.precision`` (``approximators.py:271-277``): (W, f = K a)."""
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    f = K @ np.asarray(a, dtype=dt)
    W = -lik_terms(prob.likelihood, f, prob.y, sig, cut, dt)["d2"]
    return W, f


def objective(prob: Problem, theta, tol=1e-5, maxiter=100, dtype=np.float64, a=None, K=None):
    """``LaplaceGP.objective`` -> ``objective_LA`` (``Laplace.py:12-30``).

    -sum log p(f) + 1/2 f^T a + sum log diag chol(K + diag(1/W)) + 1/2 sum log W
    at the Newton fixed point a.  Returns (value, a, iterations).
    """
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    it = None
    if a is None:
        a, it = newton_weight(prob, theta, tol, maxiter, dt, K=K)
    _, _, sig, cut = prob.split(theta)
    f = K @ a
    t = lik_terms(prob.likelihood, f, prob.y, sig, cut, dt)
    W = -t["d2"]
    with np.errstate(all="ignore"):
        try:
            Lc = np.linalg.cholesky(K + np.diag(dt(1) / W))
            logdet = np.sum(np.log(np.diag(Lc)), dtype=dt)
        except np.linalg.LinAlgError:
            logdet = dt(np.nan)
        val = (-np.sum(t["logp"], dtype=dt) + dt(0.5) * (f @ a) + logdet
               + dt(0.5) * np.sum(np.log(W), dtype=dt))
    return dt(val), a, it


def value_and_grad(prob: Problem, theta, tol=1e-5, maxiter=100, dtype=np.float64,
                   block=1024):
    """``Approximator.value_and_grad`` (``approximators.py:132-134``).

    The gradient of ``objective_LA`` at a*(theta) through the implicit layer
    of ``solvers.py:28-64``: the explicit partials (a held fixed) plus
    u^T dF/dtheta with u = (I + K W)^-1 zbar, zbar = dPsi/da
    (``fixed_point_layer_bwd``, ``solvers.py:52-64``, whose linear fixed point
    u = K diag(d2) u + zbar is solved here directly).  With R = (K + W^-1)^-1,
    Sigma = (K^-1 + W)^-1 and s = 1/2 diag(Sigma) * d3:

      zbar      = K (a - d1 - s)
      prior k   : 1/2 tr(R dK_k) + c^T dK_k a,   c = a/2 - d1 - s - W u
      lik   l   : sum_i -dlogp_i/dl - 1/2 Sigma_ii dd2_i/dl + u_i dd1_i/dl

    Returns (value, grad (n_theta,), a, iterations).
    """
    dt = np.dtype(dtype).type
    K = _K(prob, theta, dt)
    a, it = newton_weight(prob, theta, tol, maxiter, dt, K=K)
    val, _, _ = objective(prob, theta, dtype=dt, a=a, K=K)
    ell, s, sig, cut = prob.split(theta)
    N = K.shape[0]
    f = K @ a
    t = lik_terms(prob.likelihood, f, prob.y, sig, cut, dt)
    W = -t["d2"]
    with np.errstate(all="ignore"):
        Kw = K + np.diag(dt(1) / W)
        try:
            cf = sla.cho_factor(Kw, lower=True, check_finite=False)
            R = sla.cho_solve(cf, np.eye(N, dtype=dt), check_finite=False)
        except (sla.LinAlgError, ValueError):
            R = np.full((N, N), np.nan, dtype=dt)
        # Sigma = K - K R K ; only its diagonal is needed
        KR = K @ R
        diag_sigma = np.diag(K) - np.einsum("ij,ji->i", KR, K)
        sv = dt(0.5) * diag_sigma * t["d3"]
        zbar = K @ (a - t["d1"] - sv)
        u = sla.solve(np.eye(N, dtype=dt) + K * W[None, :], zbar, check_finite=False)
        c = dt(0.5) * a - t["d1"] - sv - W * u
    nl = prob.n_lengthscales
    grad = np.zeros(prob.n_theta, dtype=np.float64)
    Rd = R.astype(np.float64)
    cd = c.astype(np.float64)
    ad = a.astype(np.float64)
    for r0 in range(0, N, block):
        rows = slice(r0, min(N, r0 + block))
        _, dKs = gram_param_derivs(prob.kernel, prob.X, ell, float(s), prob.period, rows)
        for k, dK in enumerate(dKs):
            grad[k] += 0.5 * np.sum(Rd[rows] * dK) + cd[rows] @ (dK @ ad)
    ds = diag_sigma.astype(np.float64)
    ud = u.astype(np.float64)
    grad[nl + 1] = np.sum(-t["dlogp_dsig"] - 0.5 * ds * t["dd2_dsig"] + ud * t["dd1_dsig"])
    if prob.likelihood != "gaussian":
        lo = -t["dlogp_dlo"] - 0.5 * ds * t["dd2_dlo"] + ud * t["dd1_dlo"]
        hi = -t["dlogp_dhi"] - 0.5 * ds * t["dd2_dhi"] + ud * t["dd1_dhi"]
        gc = np.zeros(prob.J + 1)
        np.add.at(gc, t["y"], lo)
        np.add.at(gc, t["y"] + 1, hi)
        gc[0] = 0.0
        gc[prob.J] = 0.0
        grad[nl + 2:] = gc
    return dt(val), grad.astype(dt), a, it


def predict(prob: Problem, theta, Xs, a, W, dtype=np.float64):
    """``Approximator.predict`` (``approximators.py:154-180``).

    mean = Kfs^T a; var = Kss - sum(Kfs * solve(Kff + diag(1/W), Kfs), 0).
    """
    dt = np.dtype(dtype).type
    ell, s, _, _ = prob.split(theta)
    Kss = gram_diag(prob.kernel, Xs, dt(s), dt)
    Kfs = gram(prob.kernel, prob.X, Xs, ell, s, prob.period, dt, prob.distance)
    K = _K(prob, theta, dt) + np.diag(dt(1) / np.asarray(W, dtype=dt))
    with np.errstate(all="ignore"):
        sol = sla.solve(K, Kfs, check_finite=False)
    var = Kss - np.einsum("ij,ij->j", Kfs, sol.astype(dt))
    mean = Kfs.T @ np.asarray(a, dtype=dt)
    return mean.astype(dt), var.astype(dt)


def predict_covariance(prob: Problem, theta, Xs, a, W, dtype=np.float64):
    """``Approximator.predict_covariance`` (``approximators.py:182-197``)."""
    dt = np.dtype(dtype).type
    ell, s, _, _ = prob.split(theta)
    Kss = gram(prob.kernel, Xs, Xs, ell, s, prob.period, dt, prob.distance)
    Kfs = gram(prob.kernel, prob.X, Xs, ell, s, prob.period, dt, prob.distance)
    K = _K(prob, theta, dt) + np.diag(dt(1) / np.asarray(W, dtype=dt))
    return (Kss - Kfs.T @ sla.solve(K, Kfs, check_finite=False)).astype(dt)


def predictive_distributions(sigma, cutpoints, mean, var, dtype=np.float64):
    """``probit_predictive_distributions`` (``utilities.py:232-249``).

    p(y=j) = Phi((b_{j+1}-mu)/s) - Phi((b_j-mu)/s), s = sqrt(var + sigma^2),
    through the guarded ``probit`` of ``utilities.py:195-229``.
    """
    dt = np.dtype(dtype).type
    mean = np.asarray(mean, dtype=dt)
    std = np.sqrt(np.asarray(var, dtype=dt) + dt(sigma) ** 2)
    cut = np.asarray(cutpoints, dtype=dt)
    J = cut.size - 1
    out = np.empty((mean.size, J), dtype=dt)
    for j in range(J):
        lo = np.where(np.isinf(cut[j]), dt(0), norm_cdf(np.where(np.isinf(cut[j]), dt(0), cut[j] - mean) / std))
        hi = np.where(np.isinf(cut[j + 1]), dt(1), norm_cdf(np.where(np.isinf(cut[j + 1]), dt(0), cut[j + 1] - mean) / std))
        out[:, j] = hi - lo
    return out


# ---------------------------------------------------------------- B form
# The GPML Algorithm 3.1 form used by the CUDA path.  In exact arithmetic it
# gives the same iterates as the LU form above (Woodbury:
# (I + W K)^-1 = I - W^1/2 B^-1 W^1/2 K, B = I + W^1/2 K W^1/2), and
# sum log diag chol(B) = sum log diag chol(K + W^-1) + 1/2 sum log W.

def newton_weight_bform(prob: Problem, theta, tol=1e-5, maxiter=100, dtype=np.float64, K=None):
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    N = K.shape[0]
    a = np.zeros(N, dtype=dt)
    it = 0
    eye = np.eye(N, dtype=dt)
    while True:
        f = K @ a
        t = lik_terms(prob.likelihood, f, prob.y, sig, cut, dt)
        W = -t["d2"]
        sw = np.sqrt(W)
        b = W * f + t["d1"]
        B = eye + sw[:, None] * K * sw[None, :]
        L = np.linalg.cholesky(B)
        v = sla.solve_triangular(L, sw * (K @ b), lower=True, check_finite=False)
        a_new = b - sw * sla.solve_triangular(L.T, v, lower=False, check_finite=False)
        err = np.sqrt(np.sum((a_new - a) ** 2, dtype=dt))
        a = a_new.astype(dt)
        it += 1
        if not (err > tol) or it >= maxiter:
            break
    return a, it


def objective_bform(prob: Problem, theta, a, dtype=np.float64):
    dt = np.dtype(dtype).type
    K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    f = K @ a
    t = lik_terms(prob.likelihood, f, prob.y, sig, cut, dt)
    sw = np.sqrt(-t["d2"])
    L = np.linalg.cholesky(np.eye(K.shape[0], dtype=dt) + sw[:, None] * K * sw[None, :])
    return dt(-np.sum(t["logp"]) + 0.5 * f @ a + np.sum(np.log(np.diag(L))))


# ---------------------------------------------------------------- Variational Bayes

def vb_map(prob: Problem, theta, w, dtype=np.float64, K=None, L_cov=None):
    """``f_VB`` (``implicit/VB.py:4-17``): (sigma^2 I + K)^-1 (K w + sigma d log p(K w)),
    the Cholesky of sigma^2 I + K solved twice (``B.cholesky_solve``)."""
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    N = K.shape[0]
    if L_cov is None:
        L_cov = np.linalg.cholesky(dt(sig) ** 2 * np.eye(N, dtype=dt) + K)
    m = K @ np.asarray(w, dtype=dt)
    t = lik_terms(prob.likelihood, m, prob.y, sig, cut, dt)
    rhs = m + dt(sig) * t["d1"]
    return sla.cho_solve((L_cov, True), rhs, check_finite=False).astype(dt)


def vb_weight(prob: Problem, theta, tol=1e-5, maxiter=100, dtype=np.float64, K=None):
    """``VBGP.weight`` (``approximators.py:332-334``): ``fwd_solver``
    (``implicit/solvers.py:7-15``, jaxopt ``FixedPointIteration``) over ``f_VB``
    from w = 0; stop once ||w_k - w_{k-1}|| <= tol or after maxiter updates.
    sigma^2 I + K does not depend on w, so it is factored once.  Returns (w, iterations)."""
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, _ = prob.split(theta)
    N = K.shape[0]
    L_cov = np.linalg.cholesky(dt(sig) ** 2 * np.eye(N, dtype=dt) + K)
    w = np.zeros(N, dtype=dt)
    it = 0
    while True:
        w_new = vb_map(prob, theta, w, dt, K, L_cov)
        err = np.sqrt(np.sum((w_new - w) ** 2, dtype=dt))
        w = w_new
        it += 1
        if not (err > tol) or it >= maxiter:
            break
    return w, it


def vb_objective(prob: Problem, theta, w, dtype=np.float64, K=None):
    """``objective_VB`` (``implicit/VB.py:20-40``) at the weight w, term by term."""
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    N = K.shape[0]
    w = np.asarray(w, dtype=dt)
    m = K @ w
    L_cov = np.linalg.cholesky(dt(sig) ** 2 * np.eye(N, dtype=dt) + K)
    L_inv = sla.solve_triangular(L_cov, np.eye(N, dtype=dt), lower=True)
    cov = sla.solve_triangular(L_cov.T, L_inv, lower=False)
    log_det_cov = -2.0 * np.sum(np.log(np.diag(L_cov)))
    trace_cov = np.sum(np.diag(cov))
    trace_posterior_cov_div_var = np.einsum("ij,ij->", K, cov)
    trace_K_inv_posterior_cov = dt(sig) ** 2 * trace_cov
    t = lik_terms(prob.likelihood, m, prob.y, sig, cut, dt)
    return dt(0.5 * trace_posterior_cov_div_var + 0.5 * trace_K_inv_posterior_cov + 0.5 * m @ w
              - N * np.log(sig) - 0.5 * log_det_cov - 0.5 * N - np.sum(t["logp"]))


def vb_objective_bform(prob: Problem, theta, w, dtype=np.float64, K=None):
    """The same objective in the form the CUDA path evaluates it, with
    B = I + K / sigma^2 = L L^T (so sigma^2 I + K = sigma^2 B):
    sum_i [1/2 rowdot_i / sigma + 1/2 (B^-1)_ii + 1/2 m_i w_i + log L_ii - 1/2 - log p_i],
    rowdot_i = sum_j (B^-1)_ij K_ij / sigma."""
    dt = np.dtype(dtype).type
    if K is None:
        K = _K(prob, theta, dt)
    _, _, sig, cut = prob.split(theta)
    N = K.shape[0]
    w = np.asarray(w, dtype=dt)
    m = K @ w
    B = np.eye(N, dtype=dt) + K / dt(sig) ** 2
    L = np.linalg.cholesky(B)
    Binv = sla.cho_solve((L, True), np.eye(N, dtype=dt))
    rowdot = np.sum(Binv * K, axis=1) / dt(sig)
    t = lik_terms(prob.likelihood, m, prob.y, sig, cut, dt)
    return dt(np.sum(0.5 * rowdot / sig + 0.5 * np.diag(Binv) + 0.5 * m * w + np.log(np.diag(L)) - 0.5
                     - t["logp"]))


def vb_value_and_grad(prob: Problem, theta, tol=1e-5, maxiter=100, dtype=np.float64):
    """``VBGP`` value and gradient: ``objective_VB`` at w*(theta) through
    ``fixed_point_layer`` (``implicit/solvers.py:28-64``) over ``f_VB``.

    With A = sigma^2 I + K, m = K w*, D2 = diag(d2(m)): the adjoint of
    ``fixed_point_layer_bwd`` is the fixed point u = K (I + sigma D2) A^-1 u
    + zbar, zbar = d obj / d w = K (w - d1) (solved here directly), v = A^-1 u,
    and, the trace terms of the objective summing to N/2 exactly,
      prior k : 1/2 tr(A^-1 dK_k) + c^T dK_k w,  c = w/2 - d1 + sigma v d2
      sigma   : (tr(B^-1) - N) / sigma - sum dlogp/dsigma
                + v^T (d1 + sigma dd1/dsigma - 2 sigma w),   B = A / sigma^2
      b (cut) : -sum dlogp/db + sigma v^T dd1/db.
    Returns (value, grad (n_theta,), w, iterations)."""
    dt = np.dtype(dtype).type
    K = _K(prob, theta, dt)
    w, it = vb_weight(prob, theta, tol, maxiter, dt, K=K)
    val = vb_objective(prob, theta, w, dt, K=K)
    ell, s, sig, cut = prob.split(theta)
    N = K.shape[0]
    m = K @ w
    t = lik_terms(prob.likelihood, m, prob.y, sig, cut, dt)
    A = dt(sig) ** 2 * np.eye(N, dtype=dt) + K
    cf = sla.cho_factor(A, lower=True, check_finite=False)
    Ainv = sla.cho_solve(cf, np.eye(N, dtype=dt), check_finite=False)
    d1, d2 = t["d1"], t["d2"]
    zbar = K @ (w - d1)
    Jt = K @ ((dt(1) + dt(sig) * d2)[:, None] * Ainv)
    u = sla.solve(np.eye(N, dtype=dt) - Jt, zbar, check_finite=False)
    v = Ainv @ u
    c = dt(0.5) * w - d1 + dt(sig) * v * d2
    nl = prob.n_lengthscales
    grad = np.zeros(prob.n_theta, dtype=np.float64)
    _, dKs = gram_param_derivs(prob.kernel, prob.X, ell, float(s), prob.period)
    for k, dK in enumerate(dKs):
        grad[k] = 0.5 * np.sum(Ainv * dK) + c @ (dK @ w)
    trBinv = float(sig) ** 2 * np.trace(Ainv)
    grad[nl + 1] = ((trBinv - N) / sig - np.sum(t["dlogp_dsig"])
                    + v @ (d1 + dt(sig) * t["dd1_dsig"] - dt(2 * sig) * w))
    if prob.likelihood != "gaussian":
        lo = -t["dlogp_dlo"] + dt(sig) * v * t["dd1_dlo"]
        hi = -t["dlogp_dhi"] + dt(sig) * v * t["dd1_dhi"]
        gc = np.zeros(prob.J + 1)
        np.add.at(gc, t["y"], lo)
        np.add.at(gc, t["y"] + 1, hi)
        gc[0] = 0.0
        gc[prob.J] = 0.0
        grad[nl + 2:] = gc
    return dt(val), grad.astype(dt), w, it
