"""bench.py's reference arm on the CPU at a small N: one JSON line with the
keys of the bench contract (the GPU arm's line is checked on the GPU machine)."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--n", "256",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["N"] == 256 and "N256" in d["config"]["workload"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def test_accuracy_check_closed_form():
    """The bench's float64 check of the headline value: its closed form is the
    oracle's objective for a Gaussian likelihood (N = 300), and a failure
    inside it is reported instead of raised."""
    import numpy as np

    sys.path.insert(0, str(ROOT))
    import bench
    from oracle import laplace as L
    from probit_gb300 import workloads as W

    p = W.regression_problem(np.random.default_rng(4), 300, 4, "eq", [0.5, 1.0, 1.5, 2.0], 1.0, 0.2)
    th = p.theta()
    v = bench.exact_gaussian_nll(p.X, p.y, th[:4], th[4], th[5])
    op = L.Problem(np.asarray(p.X, np.float64), np.asarray(p.y, np.float64), "eq", "gaussian", 4)
    v64, _, _ = L.objective(op, th, tol=1e-10)
    assert abs(v - v64) <= 1e-10 * abs(v64)
    # the check uses theta rounded to float32, as the GPU receives it
    th32 = th.astype(np.float32).astype(np.float64)
    v32 = bench.exact_gaussian_nll(p.X, p.y, th32[:4], th32[4], th32[5])
    d = bench.accuracy_check(p, v32 * (1 + 2e-5))
    assert abs(d["rel_err"] - 2e-5) < 1e-12 and d["exact_float64"] == v32

    # predictions: the closed form's own mean and variance give no error
    Xt = np.random.default_rng(5).standard_normal((200, 4)).astype(np.float32)
    p.Xtest = Xt
    _, m32, var32 = bench.exact_gaussian(p.X, p.y, th32[:4], th32[4], th32[5], Xt)
    d = bench.accuracy_check(p, v32, m32, var32, stride=4)
    assert d["predict"]["points"] == 50 and d["predict"]["mean_err_of_max"] < 1e-12
    assert d["predict"]["var_err_of_s"] < 1e-12
    # and agree with the oracle's predict at the weight and precision of the fit
    a = np.linalg.solve(L.gram("eq", p.X, p.X, th32[:4], th32[4]) + th32[5] ** 2 * np.eye(300), p.y)
    m64, v64 = L.predict(op, th32, Xt.astype(np.float64), a, np.full(300, th32[5] ** -2))
    assert np.allclose(m32, m64, rtol=1e-8, atol=1e-10) and np.allclose(var32, v64, rtol=1e-8, atol=1e-10)

    class Broken:
        def theta(self):
            raise ValueError("no data")

    assert "error" in bench.accuracy_check(Broken(), 0.0)


def test_summary_is_short_and_last():
    """The GPU arm ends its line with `summary`, a few numbers per section, so
    the tail of the output (what a reader of the run's record sees) holds
    every section's figures."""
    sys.path.insert(0, str(ROOT))
    import bench

    line = {
        "accuracy": {"rel_err": 2.3e-5, "predict": {"mean_err_of_max": 1.3e-5, "var_err_of_s": 2.7e-6}},
        "predict": {"ms": 26.7},
        "c0": {"device_ms_per_step": 3.1, "e2e_ms_per_step": 4.2, "newton_iterations": 6,
               "accuracy": {"rel_err_vs_float64": 1e-6}, "cpu_baseline": {"value": 1.5}},
        "batched": {"value": 3200.0, "e2e": {"value": 3100.0}, "plain": {"value": 500.0}, "batched_over_plain": 6.4,
                    "results_identical_to_plain": True, "cpu_baseline": {"value": 1.2}},
        "hyperopt": {"value": 600.0, "evaluation_rounds": 300, "batched_over_plain": 9.6, "e2e_over_cpu": 380.0},
        "served": {"workers": 12, "pool": 256,
                   "offered_2000_per_s": {"p50_ms": 1.0, "p99_ms": 4.0, "small_p50_ms": 0.8, "small_p99_ms": 3.0,
                                          "req_s": 1990.0, "requests": 120000, "errors": 0, "window_s": 60.0},
                   "offered_150_per_s": {"p50_ms": 0.7, "p99_ms": 3.0, "small_p50_ms": 0.6, "small_p99_ms": 2.0,
                                         "req_s": 149.0, "requests": 750, "errors": 0, "window_s": 5.0}},
        "sharded_c2": {"ranks": 1, "value": 3100.0},
    }
    s = bench.summary_of(line)
    assert set(s) == {"c1_rel_err", "c1_predict_err", "c1_predict_ms", "c0", "c2", "c3", "c4", "sharded_c2"}
    assert s["c2"]["batched_over_plain"] == 6.4 and s["c2"]["identical"] is True
    assert len(json.dumps(s)) < 1300
