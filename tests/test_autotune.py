"""The near band autotuner on the CPU: bucket choice, table round trip and
lookup (a stand-in timing function), and the task order it relies on.  Its
GPU checks are in test_zz_autotune_gpu.py."""

import pytest

from probit_gb300 import _native as N
from probit_gb300 import autotune as A


def test_tune_picks_fastest_per_bucket():
    # stand-in cost: deep bands pay on short factors, win on long ones
    def cost(n, q):
        nt = A.tiles(n)
        return nt * (1.0 + 0.2 * q) if nt < 12 else nt * (2.0 - 0.1 * min(q, 4))

    t = A.tune(cost, max_tiles=32)
    assert [(e.lo, e.hi) for e in t.entries] == [(1, 2), (3, 4), (5, 8), (9, 16), (17, 32)]
    by = {e.lo: e for e in t.entries}
    assert by[3].depth == 1 and by[5].depth == 1
    assert by[17].depth == 4
    # depths with no tile to use them are not timed
    assert max(by[1].ms) <= 1
    for e in t.entries:
        assert e.depth in e.ms and e.ms[e.depth] == min(e.ms.values())


def test_ties_keep_the_shallower_depth():
    t = A.tune(lambda n, q: 1.0, buckets=((5, 8),))
    assert t.entries[0].depth == 1


def test_table_round_trip_and_lookup(tmp_path):
    t = A.Table("GB300", [A.Entry(1, 4, 2, 256, {1: 2.0, 2: 1.0}), A.Entry(5, 64, 4, 2048, {4: 3.0})])
    p = A.save(t, tmp_path / "tune.json")
    u = A.load(p)
    assert u.device == "GB300" and len(u.entries) == 2
    assert u.entries[0].ms == {1: 2.0, 2: 1.0}
    assert u.depth(100) == 2           # 1 tile: no tile below the diagonal, depth kept
    assert u.depth(600) == 4           # 5 tiles
    assert u.depth(129) == 1           # 2 tiles: at most one tile below a diagonal
    assert u.depth(64 * 128 + 1) == 0  # no bucket: built-in rule
    with pytest.raises(ValueError):
        A.Table.from_json('{"version": 1, "entries": [{"lo": 1, "hi": 2, "depth": 0, "n": 1, "ms": {}}]}')


def test_install_and_environment(tmp_path, monkeypatch):
    t = A.Table("x", [A.Entry(1, 1 << 20, 5, 128, {5: 1.0})])
    path = A.save(t, tmp_path / "t.json")
    try:
        A.use(None)
        assert A.depth_for(5000) == 0
        A.use(t)
        assert A.depth_for(5000) == 5
        # the environment variable is read on first use only
        A._env_checked = False
        A._installed = None
        monkeypatch.setenv(A.ENV, str(path))
        assert A.depth_for(5000) == 5
    finally:
        A.use(None)


def test_builtin_rule_matches_library_order(native_lib):
    import ctypes as C

    native_lib.pgbx_dag_order.restype = C.c_int
    native_lib.pgbx_dag_order.argtypes = [C.POINTER(C.c_int32), C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                          C.c_int32, C.POINTER(C.c_int32)]
    for nt in (3, 15, 16, 40):
        arr = (C.c_int32 * 1)(nt)
        n = native_lib.pgbx_dag_order(arr, 1, 1, None, 0, None)
        a = (C.c_int32 * (4 * n))()
        b = (C.c_int32 * (4 * n))()
        native_lib.pgbx_dag_order(arr, 1, 1, None, 0, a)
        native_lib.pgbx_dag_order(arr, 1, 1, (C.c_int32 * 1)(A.builtin_depth(nt)), 0, b)
        assert a[:] == b[:]


def test_setters_reject_null_handles(native_lib):
    assert native_lib.pgb_gp_set_near_depth(None, 2) == N.PGB_EINVAL
    assert native_lib.pgb_batch_set_near_depth(None, None) == N.PGB_EINVAL
