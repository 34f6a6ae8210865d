"""Lockstep L-BFGS over many independent problems, for hyperparameter fits.

The reference fits hyperparameters one GP at a time with varz's
``minimise_l_bfgs_b`` (``examples/classification.py``, ``examples/regression.py``),
each step one ``value_and_grad`` call.  ``minimize_lockstep`` runs one L-BFGS
per problem, all advancing together: every function evaluation round is ONE
call of a batched objective for all problems (``LaplaceBatch.value_and_grad_flat``:
one launch sequence on the GPU), and the per-problem two-loop recursions and
line searches are vectorised over problems on the host.

Each problem keeps its own state (history of the last ``m`` steps, step
size, convergence flag); every round passes the objective the mask of the
problems whose value is still needed (those in a line search), so a batched
objective computes only those (``LaplaceBatch.set_enabled``).  The line search
is a backtracking Armijo search (sufficient decrease c1 = 1e-4, halving);
a non-finite value counts as no decrease, so steps that leave the domain
(e.g. unordered cutpoints) are shortened.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class LockstepResult:
    x: np.ndarray          # (B, P) final points
    f: np.ndarray          # (B,) final values
    g: np.ndarray          # (B, P) final gradients
    iterations: np.ndarray  # (B,) accepted steps per problem
    evaluations: int       # batched objective calls
    converged: np.ndarray  # (B,) gradient norm below gtol
    history: list          # per evaluation round: mean f over problems


def minimize_lockstep(fg, x0, maxiter=50, m=10, gtol=1e-5, ftol=1e-7, max_ls=12, c1=1e-4, callback=None):
    """Minimise B independent smooth functions together.

    ``fg(X, mask)`` takes a (B, P) array and a (B,) boolean mask of the
    problems whose value is needed, and returns (f (B,), g (B, P)); entries
    outside the mask are ignored.  A problem stops when its gradient norm is
    at most ``gtol``, when a step lowers its value by at most ``ftol``
    relative (scipy's L-BFGS-B rule; the objective here is a float32
    computation, so the default is 1e-7), or when its line search fails.
    Returns a :class:`LockstepResult`.
    """
    x = np.array(x0, dtype=np.float64, copy=True)
    B, P = x.shape
    f, g = fg(x, np.ones(B, dtype=bool))
    f = np.asarray(f, np.float64).copy()
    g = np.asarray(g, np.float64).copy()
    evals = 1
    S = np.zeros((B, m, P))
    Y = np.zeros((B, m, P))
    rho = np.zeros((B, m))
    nhist = np.zeros(B, dtype=np.int64)      # valid history entries
    head = np.zeros(B, dtype=np.int64)       # next slot to write
    iters = np.zeros(B, dtype=np.int64)
    done = ~np.isfinite(f) | (np.linalg.norm(g, axis=1) <= gtol)
    history = [float(np.nanmean(f))]
    for _ in range(maxiter):
        active = ~done
        if not active.any():
            break
        # two-loop recursion, newest to oldest, vectorised over problems
        q = g.copy()
        alpha = np.zeros((B, m))
        for k in range(m):
            idx = (head - 1 - k) % m
            valid = (k < nhist) & active
            s_k = S[np.arange(B), idx]
            y_k = Y[np.arange(B), idx]
            r_k = rho[np.arange(B), idx]
            a = np.where(valid, r_k * np.einsum("bp,bp->b", s_k, q), 0.0)
            alpha[:, k] = a
            q -= a[:, None] * y_k
        # initial Hessian scaling gamma = s'y / y'y of the newest pair; first
        # step: 1 / ||g|| so that the first trial moves by about 1
        newest = (head - 1) % m
        s_n = S[np.arange(B), newest]
        y_n = Y[np.arange(B), newest]
        yy = np.einsum("bp,bp->b", y_n, y_n)
        sy = np.einsum("bp,bp->b", s_n, y_n)
        gnorm = np.linalg.norm(g, axis=1)
        gamma = np.where(nhist > 0, sy / np.where(yy > 0, yy, 1.0), 1.0 / np.maximum(gnorm, 1e-12))
        r = gamma[:, None] * q
        for k in reversed(range(m)):
            idx = (head - 1 - k) % m
            valid = (k < nhist) & active
            s_k = S[np.arange(B), idx]
            y_k = Y[np.arange(B), idx]
            r_k = rho[np.arange(B), idx]
            beta = np.where(valid, r_k * np.einsum("bp,bp->b", y_k, r), 0.0)
            r += (alpha[:, k] - beta)[:, None] * s_k
        d = -r
        slope = np.einsum("bp,bp->b", g, d)
        bad_dir = ~(slope < 0)
        d[bad_dir] = -g[bad_dir] / np.maximum(gnorm[bad_dir, None], 1e-12)   # restart along -g
        slope = np.einsum("bp,bp->b", g, d)
        # backtracking Armijo search, all problems in lockstep
        step = np.ones(B)
        searching = active.copy()
        f_new, g_new, x_new = f.copy(), g.copy(), x.copy()
        for _ in range(max_ls):
            xt = np.where(searching[:, None], x + step[:, None] * d, x_new)
            ft, gt = fg(xt, searching)
            evals += 1
            ft = np.asarray(ft, np.float64)
            gt = np.asarray(gt, np.float64)
            ok = searching & np.isfinite(ft) & (ft <= f + c1 * step * slope) & np.isfinite(gt).all(axis=1)
            x_new[ok], f_new[ok], g_new[ok] = xt[ok], ft[ok], gt[ok]
            searching &= ~ok
            step = np.where(searching, 0.5 * step, step)
            history.append(float(np.nanmean(np.where(ok | ~searching, f_new, f))))
            if not searching.any():
                break
        moved = active & ~searching
        done |= active & searching          # line search failed: stop this problem
        # history update
        s = x_new - x
        y = g_new - g
        sy = np.einsum("bp,bp->b", s, y)
        keep = moved & (sy > 1e-10 * np.linalg.norm(s, axis=1) * np.linalg.norm(y, axis=1))
        bi = np.nonzero(keep)[0]
        S[bi, head[bi]] = s[bi]
        Y[bi, head[bi]] = y[bi]
        rho[bi, head[bi]] = 1.0 / sy[bi]
        head[bi] = (head[bi] + 1) % m
        nhist[bi] = np.minimum(nhist[bi] + 1, m)
        small = moved & ((f - f_new) <= ftol * np.maximum(np.maximum(np.abs(f), np.abs(f_new)), 1.0))
        x, f, g = x_new, f_new, g_new
        iters += moved
        done |= (np.linalg.norm(g, axis=1) <= gtol) | small
        if callback is not None:
            callback(x, f, g)
    conv = np.linalg.norm(g, axis=1) <= gtol
    return LockstepResult(x, f, g, iters, evals, conv, history)


# ---------------------------------------------------------------- Laplace hyperparameters
class LogParams:
    """Unconstrained coordinates of ordinal-probit (or Gaussian) hyperparameters.

    u = (log l_1..l_nl, log s, log sigma_n, b_1 .. b_{J-1}) <-> theta = (l, s,
    sigma_n, -inf, b_1 .. b_{J-1}, +inf): positives log-parametrised, the
    interior cutpoints free.  ``grad_u = (x * dtheta for the logs, dtheta for
    the cutpoints)`` by the chain rule.
    """

    def __init__(self, nl, J):
        self.nl = nl
        self.J = J
        self.P = nl + 2 + max(J - 1, 0)

    def to_theta(self, u):
        u = np.atleast_2d(u)
        nl, J = self.nl, self.J
        pos = np.exp(u[:, :nl + 2])
        if J == 0:
            return pos
        inf = np.full((u.shape[0], 1), np.inf)
        return np.concatenate([pos, -inf, u[:, nl + 2:], inf], axis=1)

    def from_theta(self, theta):
        theta = np.atleast_2d(theta)
        nl, J = self.nl, self.J
        out = [np.log(theta[:, :nl + 2])]
        if J:
            out.append(theta[:, nl + 3:nl + 2 + J])
        return np.concatenate(out, axis=1)

    def grad_u(self, theta, grad_theta):
        theta = np.atleast_2d(theta)
        grad_theta = np.atleast_2d(grad_theta)
        nl, J = self.nl, self.J
        out = [theta[:, :nl + 2] * grad_theta[:, :nl + 2]]
        if J:
            out.append(grad_theta[:, nl + 3:nl + 2 + J])
        return np.concatenate(out, axis=1)


def batch_objective(batch, lp: LogParams):
    """fg(U, mask) for ``minimize_lockstep`` over a :class:`probit_gb300.LaplaceBatch`
    whose problems all share the parameter layout ``lp``: one batched
    evidence + gradient call per evaluation, computing only the masked
    problems."""
    import torch

    B = batch.B
    Pt = lp.nl + 2 + (lp.J + 1 if lp.J else 0)
    if int(batch.theta_off[-1]) != B * Pt:
        raise ValueError("every problem of the batch must have the parameter layout of `lp`")

    def fg(U, mask=None):
        theta = lp.to_theta(U)
        th = torch.from_numpy(theta.astype(np.float32).reshape(-1))
        batch.set_enabled(mask)
        v, g = batch.value_and_grad_flat(th)
        v = v.cpu().numpy().astype(np.float64)
        g = g.cpu().numpy().astype(np.float64).reshape(B, Pt)
        return v, lp.grad_u(theta, g)

    return fg
