"""Many independent Laplace GP problems evaluated together.

The reference evaluates several problems with ``vmap(value_and_grad(nelbo))``
(``README.md:238-239``, ``examples/classification.py:489-492``), which needs
every problem to share one shape.  ``LaplaceBatch`` takes problems of any
sizes, dimensions, kernels and class counts and evaluates their objectives and
gradients with one set of kernel launches (``pgb_batch_*`` in
``include/probit_gb300.h``): every kernel covers all problems, each problem
keeps its own Newton stopping rule, and the work of all problems shares the
GPU.
"""

from __future__ import annotations

import ctypes as C
import warnings

import numpy as np

from . import _native as N
from . import autotune
from ._device import require_cuda, stream_handle
from .approximators import _assign_flat_grads, _to_leaf_tensor, _zip_grads, tree_map


class LaplaceBatch:
    """A batch of ``LaplaceGP`` problems with fixed shapes.

    ``gps`` are :class:`probit_gb300.LaplaceGP` objects (data, prior,
    likelihood, tolerance, maxiter each); ``parameters`` holds one params
    pytree per problem and fixes each problem's kernel composition,
    lengthscale count and class count.  Data are packed and uploaded once;
    :meth:`set_data` replaces them.
    """

    def __init__(self, gps, parameters):
        import torch

        self.gps = list(gps)
        if not self.gps:
            raise ValueError("a batch needs at least one problem")
        if len(parameters) != len(self.gps):
            raise ValueError("one params pytree per problem")
        self.B = len(self.gps)
        self.descs = (N.Desc * self.B)()
        self.keys = []
        for b, (gp, p) in enumerate(zip(self.gps, parameters)):
            _, key = gp._theta(p)
            kind, nl, period, J = key
            self.descs[b] = N.Desc(gp.N, gp.D, kind, nl, period, gp.mode, J, gp.tolerance, gp.maxiter, 0)
            self.keys.append(key)
        self.lib = N.load()
        self.device = require_cuda()
        h = C.c_void_p()
        N.check(self.lib.pgb_batch_create(self.descs, self.B, C.byref(h)), "pgb_batch_create")
        self.h = h
        depths = [autotune.depth_for(d.n) for d in self.descs]
        if any(depths):
            N.check(self.lib.pgb_batch_set_near_depth(self.h, (C.c_int32 * self.B)(*depths)),
                    "pgb_batch_set_near_depth")
        xo = (C.c_int64 * (self.B + 1))()
        yo = (C.c_int64 * (self.B + 1))()
        to = (C.c_int64 * (self.B + 1))()
        N.check(self.lib.pgb_batch_layout(self.h, xo, yo, to), "pgb_batch_layout")
        self.x_off = np.array(xo[:], dtype=np.int64)
        self.y_off = np.array(yo[:], dtype=np.int64)
        self.theta_off = np.array(to[:], dtype=np.int64)
        self.values = torch.empty(self.B, dtype=torch.float32, device=self.device)
        self.grads = torch.empty(int(self.theta_off[-1]), dtype=torch.float32, device=self.device)
        self.set_data([gp.data for gp in self.gps])

    # -- data -----------------------------------------------------------------
    def pack_data(self, datas):
        """Host (X_packed float32, y_packed int32 bits) for a list of (X, y)."""
        X = np.empty(int(self.x_off[-1]), dtype=np.float32)
        y = np.empty(int(self.y_off[-1]), dtype=np.int32)
        for b, (Xb, yb) in enumerate(datas):
            Xb = np.asarray(Xb.detach().cpu() if hasattr(Xb, "detach") else Xb, dtype=np.float32)
            yb = np.asarray(yb.detach().cpu() if hasattr(yb, "detach") else yb)
            d = self.descs[b]
            if Xb.shape != (d.n, d.d):
                raise ValueError(f"problem {b}: X has shape {Xb.shape}, expected {(d.n, d.d)}")
            X[self.x_off[b]:self.x_off[b + 1]] = Xb.reshape(-1)
            if d.likelihood == N.LIK_GAUSSIAN:
                y[self.y_off[b]:self.y_off[b + 1]] = yb.astype(np.float32).reshape(-1).view(np.int32)
            else:
                y[self.y_off[b]:self.y_off[b + 1]] = yb.astype(np.int32).reshape(-1)
        return X, y

    def set_data(self, datas=None, packed=None):
        """Upload the problems' data (list of (X, y), or pre-packed host/device arrays)."""
        import torch

        if packed is None:
            packed = self.pack_data(datas)
        X, y = packed
        Xd = torch.as_tensor(X)
        yd = torch.as_tensor(y)
        # the C-ABI reads exactly the packed totals of pgb_batch_layout
        if Xd.numel() != int(self.x_off[-1]) or Xd.dtype != torch.float32:
            raise ValueError(f"packed X must be {int(self.x_off[-1])} float32 values")
        if yd.numel() != int(self.y_off[-1]) or yd.element_size() != 4:
            raise ValueError(f"packed y must be {int(self.y_off[-1])} 4-byte values")
        self.Xd = Xd.to(self.device, non_blocking=True).reshape(-1).contiguous()
        self.yd = yd.to(self.device, non_blocking=True).reshape(-1).contiguous()

    # -- hyperparameters --------------------------------------------------------
    def pack_theta(self, parameters, sources=None):
        """Flat float64 theta of every problem (torch, autograd-connected) and the
        packed vector; appends each problem's theta sources (the objects its
        parts were taken from, see LaplaceGP._theta) to `sources` if given."""
        import torch

        thetas = []
        for b, (gp, p) in enumerate(zip(self.gps, parameters)):
            if sources is None:
                t, key = gp._theta(p)
            else:
                t, key, src = gp._theta(p, sources=True)
                sources.append(src)
            if key != self.keys[b]:
                raise ValueError(f"problem {b}: parameters changed the problem's shape {self.keys[b]} -> {key}")
            thetas.append(t)
        return thetas, torch.cat([t.detach() for t in thetas])

    # -- evaluation ---------------------------------------------------------------
    def set_enabled(self, mask=None, stream=None):
        """Evaluate only the problems where `mask` is true (None: all).  The
        others keep the values and gradients of their last evaluation."""
        import torch

        m = np.ones(self.B, dtype=np.int32) if mask is None else np.asarray(mask, dtype=bool).astype(np.int32)
        if m.shape != (self.B,):
            raise ValueError(f"mask must have {self.B} entries")
        self._enabled = torch.from_numpy(m).to(self.device)
        s = stream if stream is not None else stream_handle(self.device)
        N.check(self.lib.pgb_batch_set_enabled(self.h, self._enabled.data_ptr(), s), "pgb_batch_set_enabled")

    def value_and_grad_flat(self, theta_packed, stream=None):
        """(values (B,), grads (packed like theta)) as CUDA tensors; enqueued on the stream."""
        import torch

        td = torch.as_tensor(theta_packed).to(self.device, dtype=torch.float32).contiguous()
        if td.numel() != int(self.theta_off[-1]):
            raise ValueError(f"theta has {td.numel()} entries, the batch needs {int(self.theta_off[-1])}")
        s = stream if stream is not None else stream_handle(self.device)
        N.check(self.lib.pgb_batch_value_and_grad(self.h, self.Xd.data_ptr(), self.yd.data_ptr(), td.data_ptr(),
                                                  self.values.data_ptr(), self.grads.data_ptr(), s),
                "pgb_batch_value_and_grad")
        return self.values, self.grads

    def objective_flat(self, theta_packed, stream=None):
        import torch

        td = torch.as_tensor(theta_packed).to(self.device, dtype=torch.float32).contiguous()
        if td.numel() != int(self.theta_off[-1]):
            raise ValueError(f"theta has {td.numel()} entries, the batch needs {int(self.theta_off[-1])}")
        s = stream if stream is not None else stream_handle(self.device)
        N.check(self.lib.pgb_batch_objective(self.h, self.Xd.data_ptr(), self.yd.data_ptr(), td.data_ptr(),
                                             self.values.data_ptr(), s), "pgb_batch_objective")
        return self.values

    def objective(self):
        """params list -> negative log evidence of every problem (NumPy, (B,))."""

        def fn(parameters):
            _, packed = self.pack_theta(parameters)
            v = self.objective_flat(packed).cpu().numpy().astype(np.float64)
            self._warn()
            return v

        return fn

    def value_and_grad(self):
        """params list -> (values (B,), [gradient pytree per problem])."""

        def vg(parameters):
            import torch

            leaves = [tree_map(_to_leaf_tensor, p) for p in parameters]
            srcs = []
            with torch.no_grad():   # autograd is needed only for a transformed parametrisation
                thetas, packed = self.pack_theta(leaves, srcs)
            v, g = self.value_and_grad_flat(packed)
            v = v.cpu().numpy().astype(np.float64)
            g = g.cpu().numpy().astype(np.float64)
            self._warn()
            out = []
            for b, (t, lv, p) in enumerate(zip(thetas, leaves, parameters)):
                gb = g[self.theta_off[b]:self.theta_off[b + 1]]
                if not _assign_flat_grads(lv, srcs[b], gb):
                    t, _ = self.gps[b]._theta(lv)
                    if t.requires_grad:
                        t.backward(torch.from_numpy(gb.copy()))
                out.append(_zip_grads(lv, p))
            return v, out

        return vg

    def status(self):
        """Per-problem (code, iterations, notpd_col, converged) of the last evaluation."""
        st = (N.Status * self.B)()
        N.check(self.lib.pgb_batch_status(self.h, st, stream_handle(self.device)), "pgb_batch_status")
        return [(s.code, s.iterations, s.notpd_col, s.converged) for s in st]

    def _warn(self):
        bad = [(b, s[0]) for b, s in enumerate(self.status()) if s[0] != 0]
        if any(code == N.PGB_ETIMEOUT for _, code in bad):
            raise N.PgbError(N.PGB_ETIMEOUT, "batch")
        if bad:
            warnings.warn(f"{len(bad)} problem(s) failed numerically (first: problem {bad[0][0]}, "
                          f"{N.strerror(bad[0][1])}); their results are NaN", RuntimeWarning, stacklevel=3)

    def __del__(self):
        try:
            if self.h:
                import torch

                torch.cuda.current_stream().synchronize()
                self.lib.pgb_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass
