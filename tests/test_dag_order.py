"""The merged tile-task order of the factorisation kernel is topological.

The persistent factorisation hands tasks out in list order through one
atomic counter and a task only waits for tasks it depends on; the launch
cannot deadlock as long as every dependency comes earlier in the list.  The
list is built on the host (pgbx_dag_order returns it without a GPU), so this
is checked here for single problems and for mixed-size batches, for the
Newton-step (one right-hand-side row), factor-only and L^-T (identity
right-hand side) task lists, and for the evaluation Newton step of Gaussian
problems (the Newton row, then the L^-T rows, in one list).
"""

JOB_COUNT = 5
SLOT = {0: 0, 1: 1, 2: 2, 3: 4}   # task list -> job slot of its problems

import ctypes as C

import numpy as np
import pytest


def _order(lib, nts, kind, near=None, whole_max=0):
    lib.pgbx_dag_order.restype = C.c_int
    lib.pgbx_dag_order.argtypes = [C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.c_int32,
                                   C.POINTER(C.c_int32)]
    arr = (C.c_int32 * len(nts))(*nts)
    nr = None if near is None else (C.c_int32 * len(nts))(*([near] * len(nts)))
    n = lib.pgbx_dag_order(arr, len(nts), kind, nr, whole_max, None)
    assert n > 0
    out = (C.c_int32 * (4 * n))()
    assert lib.pgbx_dag_order(arr, len(nts), kind, nr, whole_max, out) == n
    return np.array(out[:], dtype=np.int64).reshape(n, 4)


def _deps(i, j, nt, kind):
    """Tasks (i', j') that task (i, j) waits for."""
    if i < nt:
        d = [(i, k) for k in range(j)] + [(j, k) for k in range(j)]
        if i != j:
            d.append((j, j))
        return d
    r = i - nt
    if kind == 3:                 # row tile 0: the Newton row; then identity rows r - 1
        k0 = 0 if r == 0 else r - 1
    else:
        k0 = r if kind == 2 else 0   # identity rows start at their own column
    return [(i, k) for k in range(k0, j)] + [(j, k) for k in range(k0, j)] + [(j, j)]


@pytest.mark.parametrize("near", [None, 1, 2, 4, 16])
@pytest.mark.parametrize("kind", [0, 1, 2, 3])
@pytest.mark.parametrize("nts", [[1], [2], [5], [17], [3, 1, 7, 2, 7], [32, 1, 1, 4, 9, 2, 16]])
def test_dag_order_topological(native_lib, nts, kind, near):
    tasks = _order(native_lib, nts, kind, near)
    pos = {}
    for t, (job, i, j, _) in enumerate(tasks):
        p = job // JOB_COUNT
        assert job % JOB_COUNT == SLOT[kind]
        key = (p, i, j)
        assert key not in pos, key
        pos[key] = t
    for p, nt in enumerate(nts):
        tri = nt * (nt + 1) // 2
        expect = tri + {0: nt, 1: 0, 2: tri, 3: nt + tri}[kind]
        assert sum(1 for k in pos if k[0] == p) == expect
        for (pp, i, j), t in pos.items():
            if pp != p:
                continue
            for dep in _deps(i, j, nt, kind):
                assert (p, *dep) in pos, (p, i, j, dep)
                assert pos[(p, *dep)] < t, ("dependency after task", p, (i, j), dep)


def test_dag_order_lookahead(native_lib):
    """The next column's diagonal is handed out before the rest of a column,
    the two tiles below a diagonal before the next diagonal."""
    tasks = _order(native_lib, [6], 1)
    seq = [(int(i), int(j)) for _, i, j, _ in tasks]
    assert seq.index((1, 1)) < seq.index((3, 0))
    assert seq.index((2, 2)) < seq.index((4, 1))
    assert seq.index((3, 3)) < seq.index((5, 2))
    assert seq.index((2, 0)) < seq.index((1, 1))
    assert seq.index((3, 1)) < seq.index((2, 2))


def test_dag_order_near_depth(native_lib):
    """With a near band of depth q the q tiles below a diagonal come before
    the next diagonal and the (q+1)-th after it."""
    for q in (1, 3, 5):
        seq = [(int(i), int(j)) for _, i, j, _ in _order(native_lib, [12], 1, q)]
        for j in range(4):
            nxt = seq.index((j + 1, j + 1))
            assert all(seq.index((j + d, j)) < nxt for d in range(1, q + 1)), (q, j)
            assert seq.index((j + q + 1, j)) > nxt, (q, j)
    arr = (C.c_int32 * 1)(12)
    assert native_lib.pgbx_dag_order(arr, 1, 1, (C.c_int32 * 1)(0), 0, None) == -1   # depth 0 is refused


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_small_problems_run_whole(native_lib, kind):
    """Problems of at most whole_max tile rows are one task (i = -1) in the
    first stage; the others keep every tile task, in the same order."""
    nts = [5, 1, 2, 3, 2]
    tasks = _order(native_lib, nts, kind, whole_max=2)
    whole = [int(job) // JOB_COUNT for job, i, _, _ in tasks if i == -1]
    assert sorted(whole) == [1, 2, 4]
    # first stage: the diagonal tile of column 0 of the large problems and the
    # whole problems, by size
    first = [(int(job) // JOB_COUNT, int(i)) for job, i, _, _ in tasks[:5]]
    assert first == [(0, 0), (3, 0), (2, -1), (4, -1), (1, -1)]
    rest = [(int(job) // JOB_COUNT, int(i), int(j)) for job, i, j, _ in tasks if i != -1]
    assert {p for p, _, _ in rest} == {0, 3}
    full = _order(native_lib, nts, kind, whole_max=0)
    kept = [(int(job) // JOB_COUNT, int(i), int(j)) for job, i, j, _ in full if int(job) // JOB_COUNT in (0, 3)]
    assert rest == kept
