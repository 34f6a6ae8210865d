"""probit_gb300.autograd.evidence on the GPU: the torch.autograd.Function
gives the value of ``value_and_grad`` and, through ``backward``, the same
gradient on the torch leaves (one native value-and-gradient call either way;
Laplace and VB)."""

import math

import numpy as np
import pytest


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
