"""Drop-in ``LaplaceGP`` backed by the sm_103a CUDA library.

Mirrors the reference class (``probit/approximators.py:213-277`` with the
shared methods of ``Approximator``, ``:16-210``): same constructor arguments,
method names, argument meanings and return tuples.  Every numerical step runs
in ``libprobit_gb300.so`` through its C-ABI; hyperparameter pytrees are mapped
to the library's flat ``theta`` vector with torch autograd, which also carries
the library's d(-log Z)/d(theta) back to arbitrary ``params`` structures.
"""

from __future__ import annotations

import ctypes as C
import math
import warnings

import numpy as np

from . import _native as N
from . import autotune
from ._device import as_device, require_cuda, stream_handle
from .kernels import KIND_EQ, KIND_EQ_PERIODIC, KIND_MATERN12, resolve
from .utilities import likelihood_mode

_KIND_CODE = {KIND_EQ: N.KERNEL_EQ, KIND_MATERN12: N.KERNEL_MATERN12, KIND_EQ_PERIODIC: N.KERNEL_EQ_PERIODIC}


# ---------------------------------------------------------------- pytrees
def tree_map(fn, tree):
    if isinstance(tree, tuple):
        return tuple(tree_map(fn, t) for t in tree)
    if isinstance(tree, list):
        return [tree_map(fn, t) for t in tree]
    if isinstance(tree, dict):
        return {k: tree_map(fn, v) for k, v in tree.items()}
    return fn(tree)


def tree_leaves(tree, out=None):
    out = [] if out is None else out
    if isinstance(tree, (tuple, list)):
        for t in tree:
            tree_leaves(t, out)
    elif isinstance(tree, dict):
        for k in tree:
            tree_leaves(tree[k], out)
    else:
        out.append(tree)
    return out


def _to_leaf_tensor(x):
    import torch

    if isinstance(x, torch.Tensor):
        t = x.detach().to(device="cpu", dtype=torch.float64).clone()
    else:
        t = torch.as_tensor(np.asarray(x, dtype=np.float64))
    return t.requires_grad_(True)


def _vector_of_n(t, n, name):
    """`t` as a flat vector of n entries (the C-ABI reads exactly n)."""
    t = t.reshape(-1)
    if t.numel() != n:
        raise ValueError(f"{name} must have N = {n} entries, got {t.numel()}")
    return t


def _assign_flat_grads(leaves, srcs, flat):
    """Write slices of a flat theta gradient straight into the ``.grad`` of
    the leaf tensors, when every part of theta is one of the leaves itself
    (``srcs``: (object, offset, size) of the lengthscales, the signal
    variance, the noise std and the cutpoints, as ``_theta(sources=True)``
    gives them) — the usual ``((l, s), (sigma, cutpoints))`` pytree.  Returns
    False, writing nothing, when some part was computed from the leaves (a
    transformed parametrisation); the caller then back-propagates through
    theta with autograd, which gives the same gradients."""
    import torch

    ids = {id(t): t for t in tree_leaves(leaves) if isinstance(t, torch.Tensor)}
    plan = []
    for obj, off, n in srcs:
        t = ids.get(id(obj))
        if t is None or t.numel() != n:
            return False
        plan.append((t, off, n))
    for t, off, n in plan:
        g = torch.from_numpy(np.array(flat[off:off + n], dtype=np.float64)).reshape(t.shape)
        t.grad = g if t.grad is None else t.grad + g
    return True


def _grad_like(t, orig):
    g = t.grad
    if g is None:
        g = np.zeros(tuple(t.shape))
    else:
        g = g.numpy()
    if np.ndim(orig) == 0 and not hasattr(orig, "shape"):
        return float(g)
    return g


class LaplaceGP:
    """A GP posterior approximation using the Laplace approximation.

    ``data = (X (N, D), y (N,))``; ``prior(params[0])`` returns a kernel built
    from :mod:`probit_gb300.kernels`; ``log_likelihood`` is one of the
    likelihoods of :mod:`probit_gb300.utilities` (or the reference's own
    ``probit.utilities`` functions, recognised by name).  ``params =
    (prior_params, likelihood_params)`` with ``likelihood_params = (sigma,)``
    for the Gaussian and ``(sigma, cutpoints[J+1])`` for the ordinal probit.

    Outputs are NumPy arrays, or CUDA torch tensors when ``X`` was given as a
    torch tensor (``array_type`` overrides).  Numerical failures give NaN as in
    the reference; :meth:`last_status` reports them.
    """

    def __repr__(self):
        return "LaplaceGP"

    def __init__(self, data, prior, log_likelihood, grad_log_likelihood=None,
                 hessian_log_likelihood=None, tolerance=1e-5, maxiter=100, array_type=None):
        self.tolerance = float(tolerance)
        self.maxiter = int(maxiter)
        self.prior = prior
        self.log_likelihood = log_likelihood
        self.mode = likelihood_mode(log_likelihood, grad_log_likelihood, hessian_log_likelihood)
        self._handles = {}
        self._last = None
        self._array_type = array_type
        self.data = data

    # -- data ---------------------------------------------------------------
    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, data):
        X, y = data
        shape = tuple(X.shape)
        if len(shape) != 2:
            raise ValueError(f"X must be (N, D), got {shape}")
        self.N, self.D = int(shape[0]), int(shape[1])
        if self.D > N.MAX_D:
            raise NotImplementedError(f"D = {self.D} > {N.MAX_D} input dimensions")
        if tuple(y.shape)[:1] != (self.N,):
            raise ValueError("y must have N entries")
        if getattr(self, "_shape", None) not in (None, (self.N, self.D)) and self._handles:
            # native handles are sized for the old shape; work still queued on
            # the caller's streams may use them, so the device is drained first
            import torch

            if torch.cuda.is_available():
                torch.cuda.synchronize()
            self._handles.clear()
        self._shape = (self.N, self.D)
        self._data = data
        self._Xd = None
        self._yd = None
        self._last = None
        if self._array_type is None:
            self._out_torch = type(X).__module__.startswith("torch")
        else:
            self._out_torch = self._array_type == "torch"

    def _device_data(self):
        import torch

        if self._Xd is None:
            X, y = self._data
            self._Xd = as_device(X, torch.float32)
            if self.mode == N.LIK_GAUSSIAN:
                self._yd = as_device(y, torch.float32).reshape(-1)
            else:
                yy = y if isinstance(y, torch.Tensor) else np.asarray(y).astype(np.int32)
                self._yd = as_device(yy, torch.int32).reshape(-1)
        return self._Xd, self._yd

    # -- hyperparameters ----------------------------------------------------
    def _theta(self, params, sources=False):
        """Flat theta (float64 torch, autograd-connected to the leaves) and the
        shape key; with `sources`, also the (object, offset, size) each part of
        theta was taken from (for _assign_flat_grads)."""
        import torch

        prior_params, lik_params = params[0], params[1]
        spec = resolve(self.prior(prior_params))

        def t64(x):
            if isinstance(x, torch.Tensor):
                return x.to(torch.float64).reshape(-1)
            return torch.as_tensor(np.asarray(x, dtype=np.float64)).reshape(-1)

        ell = t64(spec.lengthscale)
        nl = ell.numel()
        if nl not in (1, self.D):
            raise ValueError(f"{nl} lengthscales for D = {self.D}")
        s = t64(spec.variance)
        if s.numel() != 1:
            raise ValueError("the signal variance must be a scalar")
        lp = lik_params if isinstance(lik_params, (tuple, list)) else (lik_params,)
        sigma = t64(lp[0])
        parts = [ell, s, sigma]
        J = 0
        if self.mode != N.LIK_GAUSSIAN:
            if len(lp) < 2:
                raise ValueError("probit likelihood_parameters must be (noise_std, cutpoints)")
            cut = t64(lp[1])
            J = cut.numel() - 1
            parts.append(cut)
        theta = torch.cat(parts)
        period = float(spec.period) if spec.period is not None else 1.0
        key = (_KIND_CODE[spec.kind], nl, period, J)
        if sources:
            srcs = [(spec.lengthscale, 0, nl), (spec.variance, nl, 1), (lp[0], nl + 1, 1)]
            if J:
                srcs.append((lp[1], nl + 2, J + 1))
            return theta, key, srcs
        return theta, key

    def _handle(self, key):
        gp = self._handles.get(key)
        if gp is not None:
            gp.gen += 1
            return gp
        kind, nl, period, J = key
        desc = N.Desc(self.N, self.D, kind, nl, period, self.mode, J, self.tolerance, self.maxiter, 0)
        lib = N.load()
        h = C.c_void_p()
        N.check(lib.pgb_gp_create(desc, C.byref(h)), "pgb_gp_create")
        gp = _Handle(lib, h, desc)
        self._handles[key] = gp
        depth = autotune.depth_for(self.N)
        if depth:
            N.check(lib.pgb_gp_set_near_depth(h, depth), "pgb_gp_set_near_depth")
        return gp

    def _theta_dev(self, theta64):
        import torch

        return theta64.detach().to(dtype=torch.float32, device=require_cuda()).contiguous()

    def _out(self, t):
        return t if self._out_torch else t.cpu().numpy()

    def last_status(self):
        """(code, iterations, notpd_col, converged) of the most recent operation."""
        if self._last_handle is None:
            return None
        return self._last_handle.status()

    _last_handle = None

    def _after(self, gp, where):
        self._last_handle = gp
        st = gp.status()
        if st[0] == N.PGB_ETIMEOUT:
            raise N.PgbError(st[0], where)
        if st[0] != 0:
            warnings.warn(f"{where}: {N.strerror(st[0])}; results contain NaN", RuntimeWarning, stacklevel=3)
        return st

    # -- reference API --------------------------------------------------------
    def construct(self):
        """params, weight -> grad log p(K weight): the fixed-point map ``f_LA``."""

        def f_LA(parameters, weight):
            import torch

            theta, key = self._theta(parameters)
            gp = self._handle(key)
            X, y = self._device_data()
            td = self._theta_dev(theta)
            a = _vector_of_n(as_device(weight, torch.float32), self.N, "weight")
            W = torch.empty(self.N, dtype=torch.float32, device=td.device)
            f = torch.empty_like(W)
            s = stream_handle(td.device)
            N.check(gp.lib.pgb_precision(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), a.data_ptr(),
                                         W.data_ptr(), f.data_ptr(), s), "pgb_precision")
            d1 = torch.empty_like(W)
            N.check(gp.lib.pgb_log_likelihood(gp.desc, td.data_ptr(), f.data_ptr(), y.data_ptr(), self.N, None,
                                              d1.data_ptr(), None, None, s), "pgb_log_likelihood")
            return self._out(d1)

        return f_LA

    def objective(self):
        """params -> negative log evidence at the Newton fixed point."""

        def objective_fn(parameters):
            import torch

            theta, key = self._theta(parameters)
            gp = self._handle(key)
            X, y = self._device_data()
            td = self._theta_dev(theta)
            v = torch.empty(1, dtype=torch.float32, device=td.device)
            N.check(gp.lib.pgb_objective(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), v.data_ptr(),
                                         stream_handle(td.device)), "pgb_objective")
            out = float(v.item())
            self._after(gp, "objective")
            return out

        return objective_fn

    def value_and_grad(self):
        """params -> (negative log evidence, gradient pytree shaped like params)."""

        def vg(parameters):
            import torch

            leaves = tree_map(_to_leaf_tensor, parameters)
            with torch.no_grad():   # autograd is needed only for a transformed parametrisation
                theta, key, srcs = self._theta(leaves, sources=True)
            gp = self._handle(key)
            X, y = self._device_data()
            td = self._theta_dev(theta)
            out = torch.empty(1 + td.numel(), dtype=torch.float32, device=td.device)
            N.check(gp.lib.pgb_value_and_grad(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(),
                                              out.data_ptr(), out[1:].data_ptr(), stream_handle(td.device)),
                    "pgb_value_and_grad")
            host = out.cpu().numpy().astype(np.float64)
            self._after(gp, "value_and_grad")
            if not _assign_flat_grads(leaves, srcs, host[1:]):
                theta, _ = self._theta(leaves)
                if theta.requires_grad:
                    theta.backward(torch.from_numpy(host[1:]))
            grads = _zip_grads(leaves, parameters)
            return float(host[0]), grads

        return vg

    def weight(self, parameters):
        """Newton fixed point a* from a = 0 (``LaplaceGP.weight``)."""
        import torch

        theta, key = self._theta(parameters)
        gp = self._handle(key)
        X, y = self._device_data()
        td = self._theta_dev(theta)
        a = torch.empty(self.N, dtype=torch.float32, device=td.device)
        N.check(gp.lib.pgb_weight(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), a.data_ptr(),
                                  stream_handle(td.device)), "pgb_weight")
        self._after(gp, "weight")
        return self._out(a)

    def precision(self, weight, parameters):
        """(W, f) with f = K weight, W = -d2 log p(f) (``LaplaceGP.precision``)."""
        import torch

        theta, key = self._theta(parameters)
        gp = self._handle(key)
        X, y = self._device_data()
        td = self._theta_dev(theta)
        a = _vector_of_n(as_device(weight, torch.float32), self.N, "weight")
        W = torch.empty(self.N, dtype=torch.float32, device=td.device)
        f = torch.empty_like(W)
        N.check(gp.lib.pgb_precision(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), a.data_ptr(),
                                     W.data_ptr(), f.data_ptr(), stream_handle(td.device)), "pgb_precision")
        return self._out(W), self._out(f)

    def approximate_posterior(self, parameters):
        """(weight, precision) at the Newton fixed point."""
        import torch

        theta, key = self._theta(parameters)
        gp = self._handle(key)
        X, y = self._device_data()
        td = self._theta_dev(theta)
        a = torch.empty(self.N, dtype=torch.float32, device=td.device)
        W = torch.empty_like(a)
        N.check(gp.lib.pgb_approximate_posterior(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(),
                                                 a.data_ptr(), W.data_ptr(), stream_handle(td.device)),
                "pgb_approximate_posterior")
        self._after(gp, "approximate_posterior")
        ao, Wo = self._out(a), self._out(W)
        self._last = (ao, Wo, a, W, theta.detach().numpy().tobytes(), key, gp.gen)
        return ao, Wo

    def predict(self, X_test, parameters, weight, precision):
        """Predictive (mean (M,), variance (M,)) at X_test (``Approximator.predict``)."""
        import torch

        theta, key = self._theta(parameters)
        gp = self._handles.get(key) or self._handle(key)
        X, _ = self._device_data()
        td = self._theta_dev(theta)
        Xs = as_device(X_test, torch.float32)
        if Xs.dim() != 2 or Xs.shape[1] != self.D:
            raise ValueError(f"X_test must be (M, {self.D})")
        M = int(Xs.shape[0])
        reuse = 0
        last = self._last
        if (last is not None and weight is last[0] and precision is last[1] and key == last[5]
                and theta.detach().numpy().tobytes() == last[4] and gp.gen == last[6]):
            a, W, reuse = last[2], last[3], 1
        else:
            gp.gen += 1
            a = _vector_of_n(as_device(weight, torch.float32), self.N, "weight")
            W = _vector_of_n(as_device(precision, torch.float32), self.N, "precision")
        mean = torch.empty(M, dtype=torch.float32, device=td.device)
        var = torch.empty_like(mean)
        N.check(gp.lib.pgb_predict(gp.h, X.data_ptr(), td.data_ptr(), a.data_ptr(), W.data_ptr(),
                                   Xs.data_ptr(), M, mean.data_ptr(), var.data_ptr(), reuse,
                                   stream_handle(td.device)), "pgb_predict")
        return self._out(mean), self._out(var)

    def predict_covariance(self, X_test, parameters, weight, precision):
        """Full predictive covariance (M, M) at X_test (``Approximator.predict_covariance``,
        ``approximators.py:182-197``): K(X*, X*) - K_*^T (K + W^-1)^-1 K_*."""
        import torch

        theta, key = self._theta(parameters)
        gp = self._handles.get(key) or self._handle(key)
        X, _ = self._device_data()
        td = self._theta_dev(theta)
        Xs = as_device(X_test, torch.float32)
        if Xs.dim() != 2 or Xs.shape[1] != self.D:
            raise ValueError(f"X_test must be (M, {self.D})")
        M = int(Xs.shape[0])
        reuse = 0
        last = self._last
        if (last is not None and weight is last[0] and precision is last[1] and key == last[5]
                and theta.detach().numpy().tobytes() == last[4] and gp.gen == last[6]):
            W, reuse = last[3], 1
        else:
            gp.gen += 1
            W = _vector_of_n(as_device(precision, torch.float32), self.N, "precision")
        cov = torch.empty((M, M), dtype=torch.float32, device=td.device)
        N.check(gp.lib.pgb_predict_covariance(gp.h, X.data_ptr(), td.data_ptr(), W.data_ptr(), Xs.data_ptr(), M,
                                              cov.data_ptr(), M, reuse, stream_handle(td.device)),
                "pgb_predict_covariance")
        return self._out(cov)

    def posterior_mean(self, weight, parameters):
        """K weight (the reference's version reads an undefined name, :199-202)."""
        return self.precision(weight, parameters)[1]


class VBGP(LaplaceGP):
    """A GP posterior approximation using Variational Bayes (``VBGP``,
    ``approximators.py:280-339``).

    The weight is the fixed point of ``f_VB`` (``implicit/VB.py:4-17``),
    w <- (sigma^2 I + K)^-1 (K w + sigma d log p(K w)), iterated from w = 0
    with the stopping rule of ``fwd_solver`` (``implicit/solvers.py:7-15``);
    sigma^2 I + K = sigma^2 (I + K / sigma^2) is factored once on the device
    and every step is a Gram matvec and two triangular solves.  The objective
    is ``objective_VB`` (``implicit/VB.py:20-40``) and ``value_and_grad`` its
    gradient through the implicit layer (``implicit/solvers.py:28-64``): the
    adjoint fixed point over ``f_VB`` on the same factor.  The precision is 1 / sigma^2 at
    every point (``approximators.py:336-339``), so ``predict`` and
    ``predict_covariance`` are those of the base class with that precision.
    Same constructor, data and parameter conventions as :class:`LaplaceGP`.
    """

    def __repr__(self):
        return "VBGP"

    def construct(self):
        raise NotImplementedError("VBGP.construct: the VB map is evaluated inside pgb_vb_weight only")

    def objective(self):
        """params -> objective_VB at the VB fixed point."""

        def objective_fn(parameters):
            import torch

            theta, key = self._theta(parameters)
            gp = self._handle(key)
            X, y = self._device_data()
            td = self._theta_dev(theta)
            v = torch.empty(1, dtype=torch.float32, device=td.device)
            N.check(gp.lib.pgb_vb_objective(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), v.data_ptr(),
                                            stream_handle(td.device)), "pgb_vb_objective")
            out = float(v.item())
            self._after(gp, "objective")
            return out

        return objective_fn

    def value_and_grad(self):
        """params -> (objective_VB, gradient pytree shaped like params) through the
        implicit layer (the adjoint fixed point over f_VB)."""

        def vg(parameters):
            import torch

            leaves = tree_map(_to_leaf_tensor, parameters)
            with torch.no_grad():   # autograd is needed only for a transformed parametrisation
                theta, key, srcs = self._theta(leaves, sources=True)
            gp = self._handle(key)
            X, y = self._device_data()
            td = self._theta_dev(theta)
            out = torch.empty(1 + td.numel(), dtype=torch.float32, device=td.device)
            N.check(gp.lib.pgb_vb_value_and_grad(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(),
                                                 out.data_ptr(), out[1:].data_ptr(), stream_handle(td.device)),
                    "pgb_vb_value_and_grad")
            host = out.cpu().numpy().astype(np.float64)
            self._after(gp, "value_and_grad")
            if not _assign_flat_grads(leaves, srcs, host[1:]):
                theta, _ = self._theta(leaves)
                if theta.requires_grad:
                    theta.backward(torch.from_numpy(host[1:]))
            return float(host[0]), _zip_grads(leaves, parameters)

        return vg

    def weight(self, parameters):
        """VB fixed point w* from w = 0 (``VBGP.weight``)."""
        import torch

        theta, key = self._theta(parameters)
        gp = self._handle(key)
        X, y = self._device_data()
        td = self._theta_dev(theta)
        w = torch.empty(self.N, dtype=torch.float32, device=td.device)
        N.check(gp.lib.pgb_vb_weight(gp.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), w.data_ptr(),
                                     stream_handle(td.device)), "pgb_vb_weight")
        self._after(gp, "weight")
        return self._out(w)

    def precision(self, weight, parameters):
        """(1 / sigma^2 at every point, K weight) (``VBGP.precision``)."""
        import torch

        _, f = LaplaceGP.precision(self, weight, parameters)
        lp = parameters[1] if isinstance(parameters[1], (tuple, list)) else (parameters[1],)
        sig = float(lp[0].item() if hasattr(lp[0], "item") else lp[0])
        W = torch.full((self.N,), 1.0 / (sig * sig), dtype=torch.float32, device=require_cuda())
        return self._out(W), f

    def approximate_posterior(self, parameters):
        """(weight, precision) at the VB fixed point."""
        w = self.weight(parameters)
        W, _ = self.precision(w, parameters)
        self._last = None
        return w, W


def _zip_grads(leaves, params):
    if isinstance(params, tuple):
        return tuple(_zip_grads(l, p) for l, p in zip(leaves, params))
    if isinstance(params, list):
        return [_zip_grads(l, p) for l, p in zip(leaves, params)]
    if isinstance(params, dict):
        return {k: _zip_grads(leaves[k], params[k]) for k in params}
    return _grad_like(leaves, params)


class _Handle:
    """Owns one pgb_gp handle."""

    def __init__(self, lib, h, desc):
        self.lib = lib
        self.h = h
        self.desc = desc
        self.gen = 0   # bumped by every operation that may replace the resident factor

    def status(self):
        st = N.Status()
        N.check(self.lib.pgb_gp_status(self.h, C.byref(st), stream_handle()), "pgb_gp_status")
        return (st.code, st.iterations, st.notpd_col, st.converged)

    def __del__(self):
        try:
            if self.h:
                import torch

                torch.cuda.current_stream().synchronize()
                self.lib.pgb_gp_destroy(self.h)
                self.h = None
        except Exception:
            pass
