"""A bounded device-side wait that runs out, on the GPU, without any fault.

Every wait of the factorisation and the triangular solves on a flag that
another block releases gives up after a time limit, raises the problem's
abort word and records PGB_ETIMEOUT (the reference has no such detection:
its fixed-point loop stops silently at maxiter, implicit/solvers.py:7-15).
Here the host arranges the missing dependency: a test hook stops one
off-diagonal tile of one problem from releasing its ready flag and gives
that problem's waits a 20 ms limit.  The problem must end with
PGB_ETIMEOUT, the batch's other problems with their normal results (bitwise
those of a run without the hook), and the same batch must give every
problem's normal result once the hook is cleared.  No trap, no unbounded
spin: the waits return and the kernels finish.
"""

import ctypes as C
import math

import numpy as np
import pytest

import probit_gb300 as pg
from probit_gb300 import _native as N
from probit_gb300 import workloads as W


def _hook(lib):
    fn = lib.pgbx_batch_test_hook
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    return fn


@pytest.mark.gpu
def test_withheld_tile_times_out_one_problem(cuda_device, native_lib):
    import torch

    rng = np.random.default_rng(77)
    sizes = [500, 200, 300]          # problem 0 has 4 tile rows: tile (3, 0) feeds (3, 1..3)
    probs = [W.ordinal_problem(rng, n, 2, 3, "matern12", 1.0, 1.0, math.sqrt(0.4), [-0.5, 0.5]) for n in sizes]
    gps = [pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=1e-4) for p in probs]
    params = [p.params() for p in probs]
    batch = pg.LaplaceBatch(gps, params)
    _, theta = batch.pack_theta(params)
    hook = _hook(native_lib)

    def run():
        v, g = batch.value_and_grad_flat(theta)
        torch.cuda.synchronize()
        return v.cpu().numpy().copy(), g.cpu().numpy().copy(), batch.status()

    v_ref, g_ref, st_ref = run()
    assert all(s[0] == N.PGB_OK for s in st_ref)

    assert hook(batch.h, 0, 20000, 3, 0) == N.PGB_OK
    try:
        v, g, st = run()
        assert st[0][0] == N.PGB_ETIMEOUT, st
        for b in (1, 2):
            assert st[b][0] == N.PGB_OK and st[b][1] == st_ref[b][1]
            assert v[b].tobytes() == v_ref[b].tobytes()
            sl = slice(int(batch.theta_off[b]), int(batch.theta_off[b + 1]))
            assert g[sl].tobytes() == g_ref[sl].tobytes()
        # the host layer turns the timeout into an error
        with pytest.raises(N.PgbError) as ei:
            batch.value_and_grad()(params)
        assert ei.value.code == N.PGB_ETIMEOUT
    finally:
        assert hook(batch.h, -1, 0, -1, -1) == N.PGB_OK

    # the same batch, hook cleared: every problem's normal result again
    v2, g2, st2 = run()
    assert all(s[0] == N.PGB_OK for s in st2)
    assert v2.tobytes() == v_ref.tobytes() and g2.tobytes() == g_ref.tobytes()


@pytest.mark.gpu
def test_hook_rejects_diagonal_and_out_of_range_tiles(cuda_device, native_lib):
    rng = np.random.default_rng(3)
    p = W.ordinal_problem(rng, 300, 2, 3, "eq", 1.0, 1.0, 0.6, [-0.5, 0.5])
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=1e-4)
    batch = pg.LaplaceBatch([gp], [p.params()])
    hook = _hook(native_lib)
    assert hook(batch.h, 0, 1000, 1, 1) == N.PGB_EINVAL      # diagonal tile
    assert hook(batch.h, 0, 1000, 3, 0) == N.PGB_EINVAL      # N = 300 has 3 tile rows
    assert hook(batch.h, 1, 1000, 2, 0) == N.PGB_EINVAL      # one problem only
    assert hook(batch.h, 0, -1, 2, 0) == N.PGB_EINVAL
    assert hook(batch.h, -1, 0, -1, -1) == N.PGB_OK
