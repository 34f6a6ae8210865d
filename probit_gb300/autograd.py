"""The evidence as a differentiable torch function.

``evidence(gp, parameters)`` returns the objective (negative log evidence for
:class:`~probit_gb300.LaplaceGP`, ``objective_VB`` for
:class:`~probit_gb300.VBGP`) as a 0-d float64 tensor connected to the torch
leaves of ``parameters``: the value and the gradient with respect to the flat
hyperparameter vector come from one ``pgb_value_and_grad`` /
``pgb_vb_value_and_grad`` call (the implicit-function-theorem adjoint of the
reference's ``fixed_point_layer``, ``implicit/solvers.py:28-64``), held by a
``torch.autograd.Function`` whose backward scales that gradient by the
incoming cotangent; autograd carries it on to the leaves through the same
torch operations that built the flat vector.
"""

from __future__ import annotations

import numpy as np


def _value_and_grad_flat(gp, theta, key):
    """(value, gradient in the flat layout) of `gp` at the flat float64 `theta`."""
    import torch

    from . import _native as N
    from ._device import stream_handle
    from .approximators import VBGP

    h = gp._handle(key)
    X, y = gp._device_data()
    td = gp._theta_dev(theta)
    out = torch.empty(1 + td.numel(), dtype=torch.float32, device=td.device)
    vb = isinstance(gp, VBGP)
    fn = h.lib.pgb_vb_value_and_grad if vb else h.lib.pgb_value_and_grad
    N.check(fn(h.h, X.data_ptr(), y.data_ptr(), td.data_ptr(), out.data_ptr(), out[1:].data_ptr(),
               stream_handle(td.device)), "pgb_vb_value_and_grad" if vb else "pgb_value_and_grad")
    host = out.cpu().numpy().astype(np.float64)
    gp._after(h, "evidence")
    return host[0], host[1:]


def _function():
    import torch

    class Evidence(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, gp, key):
            value, grad = _value_and_grad_flat(gp, theta.detach(), key)
            ctx.save_for_backward(torch.as_tensor(grad, dtype=theta.dtype))
            return torch.as_tensor(value, dtype=theta.dtype)

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            return gout * grad, None, None

    return Evidence


_EVIDENCE = None


def evidence(gp, parameters):
    """The objective of `gp` at `parameters` as a differentiable 0-d tensor."""
    global _EVIDENCE
    if _EVIDENCE is None:
        _EVIDENCE = _function()
    theta, key = gp._theta(parameters)
    return _EVIDENCE.apply(theta, gp, key)
