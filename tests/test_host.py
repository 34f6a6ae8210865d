"""Host-side logic of the drop-in API (no GPU needed)."""

import math

import numpy as np
import pytest

import probit_gb300 as pg
from probit_gb300 import _native as N
from probit_gb300.approximators import LaplaceGP, tree_leaves, tree_map
from probit_gb300.kernels import EQ, Matern12, resolve
from probit_gb300.utilities import check_cutpoints, CutpointValueError, likelihood_mode


def test_kernel_composition_like_mlkernels():
    s = resolve(2.0 * EQ().stretch(0.5).periodic(0.25))
    assert (s.kind, s.lengthscale, s.variance, s.period) == ("eq_periodic", 0.5, 2.0, 0.25)
    s = resolve(Matern12().stretch(np.array([1.0, 2.0])) * 3.0)
    assert s.kind == "matern12" and s.variance == 3.0 and list(s.lengthscale) == [1.0, 2.0]
    assert resolve(EQ()).lengthscale == 1.0
    with pytest.raises(NotImplementedError):
        EQ().periodic(1.0).stretch(2.0)
    with pytest.raises(NotImplementedError):
        Matern12().periodic(1.0)
    with pytest.raises(NotImplementedError):
        EQ() + EQ()
    with pytest.raises(NotImplementedError):
        resolve(object())


def test_kernel_scaling_keeps_torch_graph():
    import torch

    ell = torch.tensor(0.7, dtype=torch.float64, requires_grad=True)
    s = torch.tensor(1.3, dtype=torch.float64, requires_grad=True)
    spec = resolve(s * EQ().stretch(ell))
    (spec.lengthscale * 2 + spec.variance).backward()
    assert ell.grad.item() == 2.0 and s.grad.item() == 1.0


def test_likelihood_mode_identity():
    assert likelihood_mode(pg.log_gaussian_likelihood) == N.LIK_GAUSSIAN
    assert likelihood_mode(pg.log_probit_likelihood) == N.LIK_PROBIT
    assert likelihood_mode(pg.log_probit_likelihood_stable, pg.grad_log_probit_likelihood,
                           pg.hessian_log_probit_likelihood) == N.LIK_PROBIT_STABLE
    with pytest.raises(NotImplementedError):
        likelihood_mode(lambda f, y, p: f)
    with pytest.raises(NotImplementedError):
        likelihood_mode(pg.log_probit_likelihood, pg.grad_log_probit_likelihood)


def test_reference_functions_recognised_by_name():
    def log_probit_likelihood(f, y, p):
        return f

    log_probit_likelihood.__module__ = "probit.utilities"
    assert likelihood_mode(log_probit_likelihood) == N.LIK_PROBIT


def test_check_cutpoints_forms():
    assert np.array_equal(check_cutpoints([-0.5, 0.5], 3), [-math.inf, -0.5, 0.5, math.inf])
    assert np.array_equal(check_cutpoints([-math.inf, -0.5, 0.5], 3), [-math.inf, -0.5, 0.5, math.inf])
    assert np.array_equal(check_cutpoints([-0.5, 0.5, math.inf], 3), [-math.inf, -0.5, 0.5, math.inf])
    with pytest.raises(CutpointValueError):
        check_cutpoints([0.5, -0.5], 3)
    with pytest.raises(ValueError):
        check_cutpoints([1.0, 2.0, 3.0, 4.0, 5.0], 3)


def test_pytree_helpers():
    t = ((1.0, np.array([1.0, 2.0])), (0.3, [4.0, {"a": 5.0}]))
    assert len(tree_leaves(t)) == 5
    d = tree_map(lambda x: np.asarray(x) * 2, t)
    assert float(d[1][1][1]["a"]) == 10.0


def test_laplacegp_theta_layout_and_key():
    X = np.zeros((5, 2), np.float32)
    y = np.zeros(5, np.int32)
    gp = LaplaceGP((X, y), lambda p: p[1] * Matern12().stretch(p[0]), pg.log_probit_likelihood)
    theta, key = gp._theta(((np.array([0.5, 0.7]), 1.5), (0.6, [-np.inf, 0.0, np.inf])))
    assert theta.tolist() == [0.5, 0.7, 1.5, 0.6, -np.inf, 0.0, np.inf]
    assert key == (N.KERNEL_MATERN12, 2, 1.0, 2)
    with pytest.raises(ValueError):
        gp._theta(((np.array([0.5, 0.7, 0.1]), 1.5), (0.6, [-np.inf, 0.0, np.inf])))
    with pytest.raises(ValueError):
        LaplaceGP((np.zeros(5), y), lambda p: EQ(), pg.log_probit_likelihood)
    assert repr(gp) == "LaplaceGP"


def test_evidence_autograd_function_carries_the_flat_gradient_to_the_leaves(monkeypatch):
    """probit_gb300.autograd.evidence: the backward scales the flat gradient of
    one value-and-gradient call by the cotangent and autograd maps it to the
    torch leaves (the native call is replaced by a stand-in on the CPU)."""
    import torch

    from probit_gb300 import autograd as AG

    calls = []

    def fake(gp, theta, key):
        t = theta.numpy()
        calls.append(key)
        g = np.where(np.isfinite(t), 2.0 * t, 0.0)
        return float(np.sum(np.where(np.isfinite(t), t * t, 0.0))), g

    monkeypatch.setattr(AG, "_value_and_grad_flat", fake)
    X = np.zeros((5, 2), np.float32)
    y = np.zeros(5, np.int32)
    gp = LaplaceGP((X, y), lambda p: p[1] * Matern12().stretch(p[0]), pg.log_probit_likelihood)
    ell = torch.tensor([0.5, 0.7], dtype=torch.float64, requires_grad=True)
    s = torch.tensor(1.5, dtype=torch.float64, requires_grad=True)
    sig = torch.tensor(0.6, dtype=torch.float64, requires_grad=True)
    cut = torch.tensor([-np.inf, 0.25, np.inf], dtype=torch.float64)
    v = AG.evidence(gp, ((torch.log(torch.exp(ell)), s), (sig, cut)))
    assert calls == [(N.KERNEL_MATERN12, 2, 1.0, 2)]
    assert abs(v.item() - (0.25 + 0.49 + 2.25 + 0.36 + 0.0625)) < 1e-12
    (3.0 * v).backward()
    assert np.allclose(ell.grad.numpy(), 3.0 * 2.0 * np.array([0.5, 0.7]))
    assert abs(s.grad.item() - 3.0 * 3.0) < 1e-12 and abs(sig.grad.item() - 3.0 * 1.2) < 1e-12


def test_check_data_and_invalid_kernel():
    X = np.zeros((3, 2))
    Xo, yo = pg.check_data((X, np.array([0, 2, 1], np.int32)))
    assert Xo is X and yo.dtype == np.int64 and yo.tolist() == [0, 2, 1]
    with pytest.raises(TypeError):
        pg.check_data((X, np.array([0.0, 1.5, 1.0])))
    e = pg.InvalidKernel("k")
    assert "is not an instance of mlkernels.Kernel" in str(e)


@pytest.mark.parametrize("case", ["isotropic", "ard", "log_param", "gaussian", "shared_leaf", "tensor_leaves"])
def test_flat_gradient_mapping_matches_autograd(case):
    """value_and_grad maps the flat gradient to the parameter pytree either by
    writing slices into the leaves (when theta's parts are the leaves
    themselves) or through torch autograd (when the prior transforms them):
    both give the same gradients, and the direct route is taken exactly when
    every part is a leaf."""
    import torch

    from probit_gb300.approximators import _assign_flat_grads, _to_leaf_tensor, _zip_grads, tree_map
    from probit_gb300.kernels import EQ

    X = np.zeros((6, 3), np.float32)
    cut = np.array([-np.inf, -0.3, 0.4, np.inf])
    lik = pg.log_probit_likelihood
    y = np.zeros(6, np.int32)
    prior = lambda p: p[1] * Matern12().stretch(p[0])  # noqa: E731
    direct = True
    if case == "isotropic":
        params = ((0.7, 1.3), (0.5, cut))
    elif case == "ard":
        params = ((np.array([0.5, 0.8, 1.1]), 1.3), (0.5, cut))
    elif case == "log_param":
        prior = lambda p: torch.exp(p[1]) * EQ().stretch(torch.exp(p[0]))  # noqa: E731
        params = ((np.log(0.7), np.log(1.3)), (0.5, cut))
        direct = False
    elif case == "gaussian":
        lik = pg.log_gaussian_likelihood
        y = np.zeros(6, np.float32)
        params = ((np.array([0.5, 0.8, 1.1]), 1.3), (0.5,))
    elif case == "shared_leaf":
        prior = lambda p: p[0] * EQ().stretch(p[0])  # noqa: E731
        params = ((0.9, 0.0), (0.5, cut))
    else:
        params = ((torch.tensor([0.5, 0.8, 1.1]), torch.tensor(1.3)), (torch.tensor(0.5), torch.tensor(cut)))
    gp = LaplaceGP((X, y), prior, lik)
    rng = np.random.default_rng(len(case))

    def mapped(use_direct):
        # the steps of value_and_grad around the native call
        leaves = tree_map(_to_leaf_tensor, params)
        with torch.no_grad():
            theta, key, srcs = gp._theta(leaves, sources=True)
        flat = rng.standard_normal(theta.numel())
        took = use_direct and _assign_flat_grads(leaves, srcs, flat)
        if not took:
            theta, _ = gp._theta(leaves)
            theta.backward(torch.from_numpy(flat))
        return took, _zip_grads(leaves, params)

    rng = np.random.default_rng(7)
    took, fast = mapped(True)
    rng = np.random.default_rng(7)
    _, slow = mapped(False)
    assert took == direct
    fl = [np.asarray(g, np.float64) for g in pg.approximators.tree_leaves(fast)]
    sl = [np.asarray(g, np.float64) for g in pg.approximators.tree_leaves(slow)]
    assert len(fl) == len(sl)
    for a, b in zip(fl, sl):
        assert a.shape == b.shape and np.allclose(a, b, rtol=1e-12, atol=0)


def test_new_data_shape_drops_handles():
    """Handles are sized for the data they were created with: data of another
    shape drops them (the same shape keeps them)."""
    X = np.zeros((5, 2), np.float32)
    y = np.zeros(5, np.int32)
    gp = LaplaceGP((X, y), lambda p: p[1] * Matern12().stretch(p[0]), pg.log_probit_likelihood)
    gp._handles[("k",)] = object()
    gp.data = (np.ones((5, 2), np.float32), y)
    assert ("k",) in gp._handles
    gp.data = (np.zeros((7, 2), np.float32), np.zeros(7, np.int32))
    assert gp._handles == {} and (gp.N, gp.D) == (7, 2)
    gp._handles[("k",)] = object()
    gp.data = (np.zeros((7, 3), np.float32), np.zeros(7, np.int32))
    assert gp._handles == {}


def test_vector_size_checks():
    """Weights and precisions handed to the C-ABI must have N entries (it
    reads exactly N)."""
    import torch

    from probit_gb300.approximators import _vector_of_n

    assert _vector_of_n(torch.zeros(2, 3), 6, "weight").shape == (6,)
    with pytest.raises(ValueError, match="weight must have N = 5"):
        _vector_of_n(torch.zeros(4), 5, "weight")


def test_serving_rejects_malformed_requests():
    """Server.submit checks what the C-ABI calls would read: a predict
    request's test points are (m >= 1, d), an evaluation's theta has the
    length the problem's descriptor gives."""
    import itertools
    import threading

    from probit_gb300 import serving as S

    srv = object.__new__(S.Server)
    srv.lock = threading.Condition()
    srv.heaps = ([], [])
    srv.seq = itertools.count()
    srv.small_n = 2048
    srv.lib = N.load()
    X = np.zeros((10, 3), np.float32)
    p = S.Problem(X, np.zeros(10, np.int32), "eq", np.array([1.0, 1.0, 0.5, -np.inf, 0.0, np.inf]), nl=1, J=2)
    srv.submit(S.Request(0.0, "predict", 0, p, Xs=np.zeros((4, 3), np.float32)))
    for bad in (np.zeros((4, 2), np.float32), np.zeros((0, 3), np.float32), np.zeros(3, np.float32)):
        with pytest.raises(ValueError):
            srv.submit(S.Request(0.0, "predict", 0, p, Xs=bad))
    srv.submit(S.Request(0.0, "vg", 0, p, theta=p.theta))
    with pytest.raises(ValueError):
        srv.submit(S.Request(0.0, "vg", 0, p, theta=p.theta[:-1]))
    with pytest.raises(ValueError):
        srv.submit(S.Request(0.0, "refit", 0, p))
    assert len(srv.heaps[0]) == 2


def test_batch_packed_data_sizes():
    """LaplaceBatch.set_data(packed=...) takes exactly the packed totals the
    C-ABI reads (float32 X, 4-byte y)."""
    import torch

    from probit_gb300.batch import LaplaceBatch

    b = object.__new__(LaplaceBatch)
    b.x_off = np.array([0, 6, 15])
    b.y_off = np.array([0, 3, 6])
    b.device = torch.device("cpu")
    b.set_data(packed=(np.zeros(15, np.float32), np.zeros(6, np.int32)))
    assert b.Xd.shape == (15,) and b.yd.shape == (6,)
    for X, y in ((np.zeros(14, np.float32), np.zeros(6, np.int32)),
                 (np.zeros(15, np.float64), np.zeros(6, np.int32)),
                 (np.zeros(15, np.float32), np.zeros(6, np.int64)),
                 (np.zeros(15, np.float32), np.zeros(5, np.int32))):
        with pytest.raises(ValueError):
            b.set_data(packed=(X, y))


def test_dlpack_arrays_of_other_frameworks_are_imported_without_copy():
    """An array that only speaks DLPack (as a JAX or CuPy array does) becomes a
    torch view of the same memory; torch tensors, NumPy arrays and plain
    Python values are left to the usual conversions."""
    import torch

    from probit_gb300._device import from_dlpack_or_none

    class Foreign:
        def __init__(self, t):
            self._t = t

        def __dlpack__(self, stream=None, **kw):
            return self._t.__dlpack__()

        def __dlpack_device__(self):
            return self._t.__dlpack_device__()

    base = torch.arange(6, dtype=torch.float32)
    v = from_dlpack_or_none(Foreign(base))
    assert v is not None and v.data_ptr() == base.data_ptr() and torch.equal(v, base)
    assert from_dlpack_or_none(base) is None
    assert from_dlpack_or_none(np.zeros(3)) is None
    assert from_dlpack_or_none([1.0, 2.0]) is None

    class Broken:
        def __dlpack__(self, stream=None, **kw):
            raise BufferError("no export")

        def __dlpack_device__(self):
            return (1, 0)

    assert from_dlpack_or_none(Broken()) is None


def test_serving_work_queue_setting():
    """The server asks for one hardware work queue per stream (two per
    worker, 8..32) before the CUDA context exists, leaves an explicit setting
    alone, and after the context exists only warns when too few were set."""
    from probit_gb300.serving import work_queue_setting

    assert work_queue_setting(12, None, False) == ("24", None)
    assert work_queue_setting(40, None, False) == ("32", None)
    assert work_queue_setting(2, None, False) == ("8", None)
    assert work_queue_setting(12, "16", False) == (None, None)       # the user's choice stands
    assert work_queue_setting(12, "32", True) == (None, None)
    for current in (None, "8", "bogus"):
        setting, warning = work_queue_setting(12, current, True)
        assert setting is None and "share a hardware queue" in warning
