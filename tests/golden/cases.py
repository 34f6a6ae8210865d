"""Seeded parity cases shared by the fixture generator and the tests.

Each case is a small problem (the oracle finishes it in well under a second)
covering one kernel family x likelihood x lengthscale layout, plus edge
shapes (N not a multiple of the 128-row tile, N = 1, one class boundary).

Tolerances: in float32 the Newton step ||a_k - a_{k-1}||_2 stalls at a
rounding floor of about 1e-6 ||a|| (8e-6 .. 4e-4 for these cases), so the
reference's default 1e-5 can sit on the floor and turn a 5-step fit into 100
iterations of noise.  The cases use a tolerance well above the floor, where
float32 and float64 stop at the same iteration.
"""

import math

import numpy as np

from probit_gb300 import workloads as W

# name -> (kind, likelihood, N, D, J, ARD, seed, tolerance, n_test)
CASES = {
    "ordinal_matern12_n200": ("matern12", "probit", 200, 2, 3, False, 10, 1e-4, 60),
    "ordinal_eq_ard_n300": ("eq", "probit", 300, 3, 4, True, 11, 1e-4, 40),
    "ordinal_periodic_n130": ("eq_periodic", "probit", 130, 1, 3, False, 12, 1e-4, 30),
    "ordinal_stable_matern12_n257": ("matern12", "probit_stable", 257, 3, 5, False, 13, 1e-4, 50),
    "ordinal_binary_eq_n90": ("eq", "probit", 90, 1, 2, False, 14, 1e-4, 20),
    "gauss_eq_ard_n400": ("eq", "gaussian", 400, 4, 0, True, 15, 1e-2, 64),
    "gauss_periodic_n64": ("eq_periodic", "gaussian", 64, 1, 0, False, 16, 1e-3, 32),
    "gauss_matern12_n1": ("matern12", "gaussian", 1, 2, 0, False, 17, 1e-5, 3),
}


def make(name):
    """(workloads.Problem, theta float64, tolerance) for a case."""
    kind, lik, N, D, J, ard, seed, tol, n_test = CASES[name]
    rng = np.random.default_rng(seed)
    ell = np.linspace(0.6, 1.4, D) if ard else 0.9
    if lik == "gaussian":
        p = W.regression_problem(rng, N, D, kind, ell, 1.2, 0.3, n_test=n_test)
    else:
        interior = [0.0] if J == 2 else list(np.linspace(-1.0, 1.0, J - 1))
        p = W.ordinal_problem(rng, N, D, J, kind, ell, 1.1, math.sqrt(0.4), interior, n_test=n_test)
    # fit with hyperparameters a little away from the generating ones
    p.lengthscale = np.atleast_1d(np.asarray(ell, dtype=np.float64)) * 1.15
    p.variance = 0.95 * p.variance
    return p, p.theta(), tol


def oracle_problem(p, lik):
    from oracle import laplace as L

    return L.Problem(p.X.astype(np.float64), p.y, p.kernel, lik, p.lengthscale.size, p.period, p.J)
