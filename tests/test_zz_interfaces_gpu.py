"""Interfaces layered over the C-ABI, on the GPU: the DLPack entry points
give the bits of the pointer entry points on the same data, and
probit_gb300.autograd.evidence (a torch.autograd.Function) gives the value
of value_and_grad and, through backward, the same gradient on the torch
leaves (Laplace and VB).  Files named test_zz_* are collected after the
core parity suite."""

import ctypes as C
import math

import numpy as np
import pytest

from probit_gb300 import _native as N


@pytest.mark.gpu
def test_dlpack_calls_match_pointer_calls(native_lib, cuda_device):
    import torch

    import probit_gb300 as pg
    from probit_gb300 import workloads as W

    n, d, J = 300, 2, 3
    p = W.ordinal_problem(np.random.default_rng(11), n, d, J, "matern12", 0.9, 1.1, 0.6, [-0.5, 0.5])
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=1e-4)
    value, _ = gp.value_and_grad()(p.params())
    h = list(gp._handles.values())[0]
    desc = N.Desc()
    N.check(native_lib.pgb_gp_desc(h.h, C.byref(desc)), "pgb_gp_desc")
    assert (desc.n, desc.d, desc.j) == (n, d, J)
    nth = native_lib.pgb_theta_size(C.byref(desc))
    theta = torch.tensor(p.theta().astype(np.float32), device=cuda_device)
    assert theta.numel() == nth
    Xd = torch.tensor(np.asarray(p.X, np.float32), device=cuda_device)
    yd = torch.tensor(np.asarray(p.y, np.int32), device=cuda_device)
    stream = torch.cuda.current_stream().cuda_stream
    out = {}
    for mode in ("pointer", "dlpack"):
        v = torch.full((1,), float("nan"), device=cuda_device)
        g = torch.full((nth,), float("nan"), device=cuda_device)
        if mode == "pointer":
            N.check(native_lib.pgb_value_and_grad(h.h, Xd.data_ptr(), yd.data_ptr(), theta.data_ptr(),
                                                  v.data_ptr(), g.data_ptr(), stream), "pgb_value_and_grad")
        else:
            caps = [N.dlpack_tensor(t) for t in (Xd, yd, theta, v, g)]
            N.check(native_lib.pgb_dl_value_and_grad(h.h, *[a for _, a in caps], stream), "pgb_dl_value_and_grad")
        torch.cuda.synchronize()
        out[mode] = (v.cpu().numpy(), g.cpu().numpy())
    assert np.array_equal(out["pointer"][0], out["dlpack"][0])
    assert np.array_equal(out["pointer"][1], out["dlpack"][1])
    assert np.isclose(out["dlpack"][0][0], value, rtol=1e-6)
    # a wrong label dtype is refused before anything is enqueued
    caps = [N.dlpack_tensor(t) for t in (Xd, yd.float(), theta, v, g)]
    assert native_lib.pgb_dl_value_and_grad(h.h, *[a for _, a in caps], stream) == N.PGB_EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("vb", [False, True])
def test_evidence_matches_value_and_grad(cuda_device, vb):
    import torch

    import probit_gb300 as pg
    from probit_gb300 import autograd as AG
    from probit_gb300 import workloads as W

    p = W.ordinal_problem(np.random.default_rng(21), 250, 2, 3, "eq", 0.8, 1.2, math.sqrt(0.4), [-0.5, 0.5])
    cls = pg.VBGP if vb else pg.LaplaceGP
    gp = cls((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=1e-4)
    v_ref, g_ref = gp.value_and_grad()(p.params())
    ell = torch.tensor(float(p.lengthscale[0]), dtype=torch.float64, requires_grad=True)
    s = torch.tensor(float(p.variance), dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(float(p.noise_std), dtype=torch.float64, requires_grad=True)
    cut = torch.tensor(np.asarray(p.cutpoints, np.float64))
    v = AG.evidence(gp, ((ell, s), (sig, cut)))
    (2.0 * v).backward()
    assert v.item() == v_ref
    for leaf, ref in ((ell, g_ref[0][0]), (s, g_ref[0][1]), (sig, g_ref[1][0])):
        assert np.isclose(leaf.grad.item(), 2.0 * float(np.asarray(ref)), rtol=1e-12, atol=0), (leaf.grad, ref)
