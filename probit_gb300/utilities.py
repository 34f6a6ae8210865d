"""Likelihoods of the Laplace path, evaluated by the CUDA library.

The names mirror the reference's ``probit/utilities.py`` so that code written
against it selects the same model:

* :func:`log_gaussian_likelihood` — ``utilities.py:60-61``
* :func:`log_probit_likelihood` — ``utilities.py:56-57`` (log(Z + 1e-10),
  Z through erf; derivatives as JAX autodiff gives them)
* :func:`log_probit_likelihood_stable` — the same ordinal model with log Z
  evaluated through erfcx (finite in the far tails)
* :func:`grad_log_probit_likelihood` / :func:`hessian_log_probit_likelihood`
  — analytic derivatives (``utilities.py:151-192`` in the reference); here
  they are the stable-mode derivatives and may be passed to ``LaplaceGP``
  together with :func:`log_probit_likelihood_stable`.

Each function takes arrays (f, y, likelihood_parameters) and returns per-point
values computed on the GPU (``pgb_log_likelihood``).
"""

from __future__ import annotations

import math

import numpy as np

from . import _native as N
from ._device import as_device, like_input, stream_handle

__all__ = [
    "log_gaussian_likelihood", "log_probit_likelihood", "log_probit_likelihood_stable",
    "grad_log_probit_likelihood", "hessian_log_probit_likelihood", "likelihood_mode",
    "check_cutpoints", "CutpointValueError", "probit_predictive_distributions",
]


def _eval(mode, f, y, likelihood_parameters, which):
    import torch

    sigma = float(np.asarray(likelihood_parameters[0], dtype=np.float64))
    if mode == N.LIK_GAUSSIAN:
        cut = np.zeros(0)
        J = 0
        yd = as_device(y, torch.float32)
    else:
        cut = np.asarray(likelihood_parameters[1], dtype=np.float64).reshape(-1)
        J = cut.size - 1
        yd = as_device(np.asarray(y).astype(np.int32) if not isinstance(y, torch.Tensor) else y, torch.int32)
    fd = as_device(f, torch.float32).reshape(-1)
    yd = yd.reshape(-1)
    n = fd.numel()
    if yd.numel() != n:
        raise ValueError(f"y has {yd.numel()} entries, f {n}")
    theta = torch.tensor(np.concatenate([[1.0, 1.0, sigma], cut]), dtype=torch.float32, device=fd.device)
    desc = N.Desc(max(n, 1), 1, N.KERNEL_EQ, 1, 1.0, mode, J, 1e-5, 100, 0)
    outs = [torch.empty(n, dtype=torch.float32, device=fd.device) for _ in range(4)]
    ptr = [o.data_ptr() if k in which else None for k, o in enumerate(outs)]
    lib = N.load()
    N.check(lib.pgb_log_likelihood(desc, theta.data_ptr(), fd.data_ptr(), yd.data_ptr(), n, *ptr,
                                   stream_handle(fd.device)), "pgb_log_likelihood")
    res = [like_input(outs[k], f) for k in which]
    return res[0] if len(res) == 1 else tuple(res)


def probit_predictive_distributions(likelihood_parameters, posterior_mean, posterior_variance):
    """Ordinal predictive distributions (N_test, J) on the GPU
    (``probit_predictive_distributions``, ``utilities.py:232-249``):
    p(y = j) = Phi((b_{j+1} - mean) / s) - Phi((b_j - mean) / s),
    s = sqrt(variance + noise_std^2)."""
    import torch

    noise_std, cutpoints = likelihood_parameters
    cut = np.asarray(cutpoints.detach().cpu() if hasattr(cutpoints, "detach") else cutpoints,
                     dtype=np.float64).reshape(-1)
    J = cut.size - 1
    md = as_device(posterior_mean, torch.float32).reshape(-1)
    vd = as_device(posterior_variance, torch.float32, md.device).reshape(-1)
    m = md.numel()
    if vd.numel() != m:
        raise ValueError(f"posterior_variance has {vd.numel()} entries, posterior_mean {m}")
    sigma = float(np.asarray(noise_std, dtype=np.float64))
    theta = torch.tensor(np.concatenate([[1.0, 1.0, sigma], cut]), dtype=torch.float32, device=md.device)
    desc = N.Desc(max(m, 1), 1, N.KERNEL_EQ, 1, 1.0, N.LIK_PROBIT, J, 1e-5, 100, 0)
    out = torch.empty((m, J), dtype=torch.float32, device=md.device)
    lib = N.load()
    N.check(lib.pgb_predictive_distributions(desc, theta.data_ptr(), md.data_ptr(), vd.data_ptr(), m,
                                             out.data_ptr(), stream_handle(md.device)),
            "pgb_predictive_distributions")
    return like_input(out, posterior_mean)


def log_gaussian_likelihood(f, y, likelihood_parameters):
    """log N(y; f, sigma^2) per point; likelihood_parameters = (sigma,)."""
    return _eval(N.LIK_GAUSSIAN, f, y, likelihood_parameters, (0,))


def log_probit_likelihood(f, y, likelihood_parameters):
    """log(Phi((b_{y+1}-f)/s) - Phi((b_y-f)/s) + 1e-10); params = (s, cutpoints)."""
    return _eval(N.LIK_PROBIT, f, y, likelihood_parameters, (0,))


def log_probit_likelihood_stable(f, y, likelihood_parameters):
    """The ordinal probit log-likelihood evaluated in log space (no +1e-10)."""
    return _eval(N.LIK_PROBIT_STABLE, f, y, likelihood_parameters, (0,))


def grad_log_probit_likelihood(f, y, likelihood_parameters):
    """d/df of :func:`log_probit_likelihood_stable`."""
    return _eval(N.LIK_PROBIT_STABLE, f, y, likelihood_parameters, (1,))


def hessian_log_probit_likelihood(f, y, likelihood_parameters):
    """d^2/df^2 of :func:`log_probit_likelihood_stable`."""
    return _eval(N.LIK_PROBIT_STABLE, f, y, likelihood_parameters, (2,))


def likelihood_mode(log_likelihood, grad_log_likelihood=None, hessian_log_likelihood=None) -> int:
    """Map the user's likelihood callables to a PGB_LIK_* mode.

    Accepts this module's functions and, by name, the reference package's
    ``probit.utilities`` functions.  Optional derivative callables must match
    the chosen model; anything else raises ``NotImplementedError``.
    """
    name = getattr(log_likelihood, "__name__", "")
    mod = getattr(log_likelihood, "__module__", "") or ""
    ours = mod == __name__
    ref = mod.startswith("probit.")
    if not (ours or ref):
        raise NotImplementedError(
            f"log_likelihood {name!r} is not one the CUDA library implements; use "
            "log_gaussian_likelihood, log_probit_likelihood or log_probit_likelihood_stable")
    modes = {"log_gaussian_likelihood": N.LIK_GAUSSIAN, "log_probit_likelihood": N.LIK_PROBIT,
             "log_probit_likelihood_stable": N.LIK_PROBIT_STABLE}
    if name not in modes:
        raise NotImplementedError(f"unsupported log_likelihood {name!r}")
    mode = modes[name]
    for fn, expect in ((grad_log_likelihood, "grad_log_probit_likelihood"),
                       (hessian_log_likelihood, "hessian_log_probit_likelihood")):
        if fn is None:
            continue
        fname = getattr(fn, "__name__", "")
        fmod = getattr(fn, "__module__", "") or ""
        if fname != expect or not (fmod == __name__ and mode == N.LIK_PROBIT_STABLE):
            raise NotImplementedError(
                f"derivative callable {fname!r} does not match the chosen likelihood; pass None "
                "(autodiff-equivalent derivatives are built in) or this module's stable-mode pair "
                "with log_probit_likelihood_stable")
    return mode


class CutpointValueError(Exception):
    """Cutpoints not in ascending order (``utilities.py:313-333``)."""

    def __init__(self, cutpoint):
        super().__init__(f"The cutpoint list or array must be in ascending order, {cutpoint} was given.")


def check_cutpoints(cutpoints, J):
    """Normalise cutpoints to the (J + 1,) form with -inf / +inf ends.

    Restates ``check_cutpoints`` (``utilities.py:251-310``): J - 1 interior
    values get both infinite ends, J values with -inf first get +inf
    appended, J values with +inf last get -inf prepended; order is checked.
    """
    c = np.asarray(cutpoints, dtype=np.float64).reshape(-1)
    if c.size == J - 1:
        c = np.concatenate([[-math.inf], c, [math.inf]])
    elif c.size == J:
        if c[-1] != math.inf:
            if c[0] != -math.inf:
                raise ValueError(
                    "Either the largest cutpoint parameter b_J is not positive infinity, or the "
                    f"smallest cutpoint parameter must b_0 is not negative infinity.(got {[c[0], c[-1]]})")
            c = np.concatenate([c, [math.inf]])
        else:
            c = np.concatenate([[-math.inf], c])
    elif c.size == J + 1:
        if c[0] != -math.inf:
            raise ValueError(f"The smallest cutpoint parameter b_0 must be negative infinity (got {c[0]})")
        if c[-1] != math.inf:
            raise ValueError(f"The largest cutpoint parameter b_J must be positive infinity (got {c[-1]})")
    else:
        raise ValueError(f"Could not recognise cutpoints shape. (shape was {c.shape})")
    if not all(c[i] <= c[i + 1] for i in range(J)):
        raise CutpointValueError(c)
    return c


def check_data(data):
    """(X, y) with integer class labels (``check_data``, ``utilities.py:252-260``):
    y must hold integers; returned as int64."""
    X, y = data
    ya = np.asarray(y)
    if not np.issubdtype(ya.dtype, np.integer):
        raise TypeError(f"t must contain only integer values (got {ya.dtype})")
    return X, ya.astype(np.int64)


class InvalidKernel(Exception):
    """A prior that is not a kernel this library evaluates (``InvalidKernel``,
    ``utilities.py:348-360``; raised by the reference's examples)."""

    def __init__(self, kernel):
        super().__init__(f"{kernel} is not an instance of mlkernels.Kernel")
