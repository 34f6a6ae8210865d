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
each trial step is first capped so that no coordinate moves by more than
``max_step`` (the L-BFGS direction can be long where the curvature
estimate is poor, and a log-parametrised coordinate moved by tens would
overflow), and a non-finite value counts as no decrease, so steps that
leave the domain are shortened.
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


def minimize_lockstep(fg, x0, maxiter=50, m=10, gtol=1e-5, ftol=1e-7, max_ls=12, c1=1e-4, max_step=2.0,
                      callback=None):
    """Minimise B independent smooth functions together.

    ``fg(X, mask)`` takes a (B, P) array and a (B,) boolean mask of the
    problems whose value is needed, and returns (f (B,), g (B, P)); entries
    outside the mask are ignored.  A problem stops when its gradient norm is
    at most ``gtol``, when a step lowers its value by at most ``ftol``
    relative (scipy's L-BFGS-B rule; the objective here is a float32
    computation, so the default is 1e-7), or when its line search fails.
    The first trial of each line search moves no coordinate by more than
    ``max_step`` (None: no cap).  Returns a :class:`LockstepResult`.
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
        # backtracking Armijo search, all problems in lockstep; the first
        # trial moves no coordinate by more than max_step
        step = np.ones(B)
        if max_step is not None:
            dmax = np.abs(d).max(axis=1)
            step = np.where(dmax > max_step, max_step / np.maximum(dmax, 1e-300), 1.0)
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

    u = (log l_1..l_nl, log s, log sigma_n, b_1, log(b_2 - b_1), ..,
    log(b_{J-1} - b_{J-2})) <-> theta = (l, s, sigma_n, -inf, b_1 .. b_{J-1},
    +inf): positives log-parametrised, the first interior cutpoint free and
    each later one the previous plus a positive increment, so every u gives
    cutpoints in increasing order (the reference's ``check_cutpoints``,
    utilities.py:263-300, rejects any other).  Log coordinates are clipped
    to [-80, 80] before the exponential (finite in float32).  The gradient in
    u follows by the chain rule (``grad_u``).
    """

    LOG_CLIP = 80.0

    def __init__(self, nl, J):
        self.nl = nl
        self.J = J
        self.P = nl + 2 + max(J - 1, 0)

    def to_theta(self, u):
        u = np.atleast_2d(np.asarray(u, np.float64))
        nl, J = self.nl, self.J
        pos = np.exp(np.clip(u[:, :nl + 2], -self.LOG_CLIP, self.LOG_CLIP))
        if J == 0:
            return pos
        inf = np.full((u.shape[0], 1), np.inf)
        if J < 2:
            return np.concatenate([pos, -inf, inf], axis=1)
        inc = np.exp(np.clip(u[:, nl + 3:], -self.LOG_CLIP, self.LOG_CLIP))
        b = np.cumsum(np.concatenate([u[:, nl + 2:nl + 3], inc], axis=1), axis=1)
        return np.concatenate([pos, -inf, b, inf], axis=1)

    def from_theta(self, theta):
        theta = np.atleast_2d(np.asarray(theta, np.float64))
        nl, J = self.nl, self.J
        out = [np.log(theta[:, :nl + 2])]
        if J >= 2:
            b = theta[:, nl + 3:nl + 2 + J]
            if np.any(np.diff(b, axis=1) <= 0):
                raise ValueError("interior cutpoints must be strictly increasing")
            out += [b[:, :1], np.log(np.diff(b, axis=1))]
        return np.concatenate(out, axis=1)

    def grad_u(self, theta, grad_theta):
        theta = np.atleast_2d(theta)
        grad_theta = np.atleast_2d(grad_theta)
        nl, J = self.nl, self.J
        out = [theta[:, :nl + 2] * grad_theta[:, :nl + 2]]
        if J >= 2:
            gb = grad_theta[:, nl + 3:nl + 2 + J]
            # b_k = b_1 + sum_{m < k} exp(v_m): d/db_1 = sum_k g_k,
            # d/dv_m = exp(v_m) sum_{k > m} g_k
            tail = np.cumsum(gb[:, ::-1], axis=1)[:, ::-1]
            b = theta[:, nl + 3:nl + 2 + J]
            out += [tail[:, :1], np.diff(b, axis=1) * tail[:, 1:]]
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
