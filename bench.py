"""Benchmark: Laplace evidence + implicit-gradient solves per second on GB300.

Workload (default, the single-GPU configuration the metric is quoted on):
Gaussian-likelihood regression, N = 8192, D = 4, X ~ N(0, I), EQ kernel with
ARD lengthscales (0.5, 1, 1.5, 2), signal variance 1, noise std 0.2, y drawn
from the GP plus noise (seeded synthetic data).  One step = one complete
evidence + gradient solve: Newton fixed point from a = 0, negative log
evidence and its gradient in the 6 hyperparameters (4 lengthscales, signal
variance, noise std).  Newton tolerance 1.0 on ||a_k - a_{k-1}||_2: the
float32 rounding floor of that norm on this data is about 0.1 (||a|| = 431),
so the reference default 1e-5 is unreachable in float32 and would run the
maximum 100 iterations.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 (torchrun, one rank per GPU): a single GP does not shard, so every rank
runs an independent replica ("scaling": "weak"); value = total solves/s.
The batched workload (1,024 ordinal problems) does shard: at N > 1 every rank
evaluates its longest-processing-time share and the results are gathered on
the host (`sharded_c2`; at N = 1 the whole batch on one GPU).

Beside the headline the line carries config 0 (`c0`), the batched, hyperopt
and serving sections, and, last, a short `summary` of each.
"""

from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

# Hardware work queues of the CUDA context (read when it is created): the
# serving section drives 24 streams at once; with the default 8 queues a
# small request's kernel can wait behind a large request's launch that only
# shares its queue.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Laplace evidence+grad solves/s"
# dram__bytes_read.sum + dram__bytes_write.sum of one N = 8192 factor-only
# launch (one-pass ncu capture, profiles/launches_gaussian_N8192_evidence_grad.md)
FACTOR_TRAFFIC_N8192 = 3.08e9 + 0.44347e9
# nominal dense TF32 tensor rate of a GB300 (TFLOP/s); a 3xTF32 product issues
# three TF32 MMAs per algorithmic one
TF32_NOMINAL_TFLOPS = 1100.0
UNIT = "solves/s"
TOL = 1.0
def config_name(n):
    return f"gaussian_eq_ard_N{n}_D4_evidence_grad"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--predict-m", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the float64 check of the headline value (a host Cholesky of N x N)")
    ap.add_argument("--batch", type=int, default=1024,
                    help="problems of the batched ordinal workload reported beside the headline (0: skip)")
    ap.add_argument("--batch-tol", type=float, default=1e-3)
    ap.add_argument("--no-plain", action="store_true", help="skip the plain one-call-per-problem comparison")
    ap.add_argument("--hyperopt", type=int, default=256,
                    help="problems of the lockstep L-BFGS hyperparameter workload (0: skip)")
    ap.add_argument("--hyperopt-steps", type=int, default=50)
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="arrival window of the serving workload at 2000 req/s (0: skip)")
    ap.add_argument("--serve-workers", type=int, default=12)
    ap.add_argument("--serve-max-large", type=int, default=5,
                    help="large (n > 2048) requests served at once (the rest of the GPU serves small ones)")
    ap.add_argument("--serve-large-blocks", type=int, default=24, help="SM share of each large request's launches")
    ap.add_argument("--serve-small-blocks", type=int, default=32,
                    help="SM share of each small request's launches (0: one block per SM)")
    ap.add_argument("--no-c0", action="store_true", help="skip the config-0 section")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1 and args.impl == "gb300":
        import torch.distributed as dist

        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ---------------------------------------------------------------- reference arm
def run_reference(args, ws, rank):
    """The reference's algorithm on the host cores (the oracle port, all threads)."""
    if rank != 0:
        return
    from oracle import laplace as L
    from probit_gb300 import workloads as Wk

    p = Wk.regression_c1(N=args.n, M=0)
    op = L.Problem(p.X, p.y.astype(np.float32), "eq", "gaussian", 4)
    theta = p.theta().astype(np.float32)
    cores = len(os.sched_getaffinity(0))
    warm = min(args.warmup, 1)
    for _ in range(warm):
        L.value_and_grad(op, theta, tol=TOL, dtype=np.float32)
    budget = 150.0
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        L.value_and_grad(op, theta, tol=TOL, dtype=np.float32)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    v = done / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": done,
        "warmup": warm, "ms_per_step": 1e3 * dt / done, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": config_name(args.n), "N": args.n, "D": 4, "tolerance": TOL},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{done} full evidence+grad solve(s) at N={args.n} with the NumPy/SciPy "
                                   "restatement of the reference algorithm (dense-Jacobian LU Newton), float32"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(args):
    """Bounded CPU sample: the oracle on one full solve (float32, all host threads)."""
    from oracle import laplace as L
    from probit_gb300 import workloads as Wk

    n = args.n
    p = Wk.regression_c1(N=n, M=0)
    op = L.Problem(p.X, p.y.astype(np.float32), "eq", "gaussian", 4)
    theta = p.theta().astype(np.float32)
    t0 = time.perf_counter()
    L.value_and_grad(op, theta, tol=TOL, dtype=np.float32)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": UNIT, "cores": len(os.sched_getaffinity(0)), "kind": "port",
            "sample": f"1 full evidence+grad solve at N={n} (NumPy/SciPy restatement of the reference "
                      f"algorithm, float32, OpenBLAS on all host threads): {dt:.1f} s"}


def eq_gram64(X1, X2, ell, s):
    """s exp(-|x1 - x2|^2 / 2) with inputs divided by the lengthscales, float64."""
    A = np.asarray(X1, np.float64) / np.asarray(ell, np.float64)
    Bm = np.asarray(X2, np.float64) / np.asarray(ell, np.float64)
    C = A @ Bm.T
    C *= -2.0
    C += np.einsum("ij,ij->i", A, A)[:, None]
    C += np.einsum("ij,ij->i", Bm, Bm)[None, :]
    np.maximum(C, 0.0, out=C)
    C *= -0.5
    np.exp(C, out=C)
    C *= s
    return C


def exact_gaussian(X, y, ell, s, sigma, Xs=None):
    """GP regression with an EQ kernel (lengthscales ell, signal variance s)
    and Gaussian noise std sigma, in float64 on the host: -log p(y) =
    1/2 y^T C^-1 y + sum log diag chol(C) + n/2 log 2 pi with C = K + sigma^2 I
    (with a Gaussian likelihood the Laplace evidence is exactly this) and, at
    test points Xs, the predictive mean K_*^T C^-1 y and latent variance
    s - diag(K_*^T C^-1 K_*).  Returns (nll, mean or None, var or None)."""
    import scipy.linalg as sla

    y = np.asarray(y, np.float64)
    C = eq_gram64(X, X, ell, s)
    C[np.diag_indices_from(C)] += sigma * sigma
    c, low = sla.cho_factor(C, lower=True, overwrite_a=True, check_finite=False)
    alpha = sla.cho_solve((c, low), y, check_finite=False)
    nll = 0.5 * float(y @ alpha) + float(np.log(np.diag(c)).sum()) + 0.5 * y.size * math.log(2 * math.pi)
    if Xs is None:
        return nll, None, None
    Ks = eq_gram64(X, Xs, ell, s)
    V = sla.solve_triangular(c, Ks, lower=True, check_finite=False)
    return nll, Ks.T @ alpha, s - np.einsum("ij,ij->j", V, V)


def exact_gaussian_nll(X, y, ell, s, sigma):
    """-log p(y) of exact_gaussian."""
    return exact_gaussian(X, y, ell, s, sigma)[0]


def accuracy_check(p, value, mean=None, var=None, stride=64):
    """The headline solve's value, and the predictive mean and variance at
    every `stride`-th test point, against the float64 closed forms (a
    size-independent property: for a Gaussian likelihood the Laplace
    evidence is the marginal likelihood and the predictions are the GP's)."""
    try:
        th = np.asarray(p.theta(), np.float32).astype(np.float64)   # the float32 theta the GPU was given
        t0 = time.perf_counter()
        Xs = None if mean is None else np.asarray(p.Xtest)[::stride]
        v64, m64, var64 = exact_gaussian(p.X, p.y, th[:4], float(th[4]), float(th[5]), Xs)
        out = {"neg_log_evidence": value, "exact_float64": v64, "rel_err": abs(value - v64) / abs(v64),
               "bar": 1e-4,
               "what": "Gaussian likelihood: the Laplace evidence is the exact GP marginal likelihood; "
                       "closed form in float64 (Cholesky of K + sigma^2 I) on the host"}
        if mean is not None:
            m = np.asarray(mean, np.float64)[::stride]
            v = np.asarray(var, np.float64)[::stride]
            out["predict"] = {"points": int(m.size), "stride": stride,
                              "mean_err_of_max": float(np.abs(m - m64).max() / np.abs(m64).max()),
                              "var_err_of_s": float(np.abs(v - var64).max() / th[4]), "bar": 1e-4}
        out["host_s"] = time.perf_counter() - t0
        return out
    except Exception as e:  # the check must not cost the bench line
        return {"error": f"{type(e).__name__}: {e}"}


# ---------------------------------------------------------------- batched workload
def launches_per_solve(iters, trace_groups=1, matvec_groups=1, factor_steps=None):
    """Kernels one evidence + gradient solve launches (each covers every problem
    of a batch): per Newton step f += K da (one per matvec group), the
    likelihood terms, the reuse check (2), the factor condition, mark_z,
    reuse marking, the two wavefront solves, the update and the stop rule (2),
    plus the factorisation in the steps that factor (`factor_steps`, default
    all: a graph IF node skips it in the others)."""
    factor_steps = iters if factor_steps is None else factor_steps
    newton = matvec_groups + 1 + 2 + 1 + 1 + 1 + 2 + 1 + 2
    epilogue = 1 + matvec_groups + 1 + 2 + 1 + 1 + 2        # activate, precision, reuse, factor, evidence
    grad = 1 + matvec_groups + 1 + matvec_groups + 1 + 1 + 1 + trace_groups + 2
    return 2 + newton * iters + factor_steps + epilogue + grad


def run_batched(args, dev):
    """The batched ordinal workload: B problems of uneven N, D, J and kernel in
    one batch, against the plain path (one single-GP call per problem)."""
    import ctypes as C

    import torch

    import probit_gb300 as pg
    from probit_gb300 import _native as N
    from probit_gb300 import workloads as Wk

    B = args.batch
    t0 = time.perf_counter()
    probs = Wk.batched_c2(B=B, device=dev)
    gen_s = time.perf_counter() - t0
    tol = args.batch_tol
    gps = [pg.LaplaceGP((q.X, q.y), q.prior(), pg.log_probit_likelihood, tolerance=tol) for q in probs]
    params = [q.params() for q in probs]
    batch = pg.LaplaceBatch(gps, params)
    _, theta = batch.pack_theta(params)
    td = theta.to(dev, torch.float32)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(3, args.warmup)):
        batch.value_and_grad_flat(td)
    torch.cuda.synchronize()
    st = batch.status()
    iters = np.array([x[1] for x in st])
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    reps = max(1, min(args.steps, 5))
    ms = []
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.value_and_grad_flat(td)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    batched_ms = statistics.median(ms)
    # end to end through LaplaceBatch: packed host inputs uploaded, values and gradients read back
    Xp, yp = batch.pack_data([(q.X, q.y) for q in probs])
    Xh, yh = torch.from_numpy(Xp).pin_memory(), torch.from_numpy(yp).pin_memory()
    th_h = theta.to(torch.float32).pin_memory()
    t0 = time.perf_counter()
    for _ in range(reps):
        batch.set_data(packed=(Xh, yh))
        v, g = batch.value_and_grad_flat(th_h)
        v.cpu(), g.cpu()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / reps
    Ns = np.array([q.N for q in probs], dtype=np.float64)
    cpu = None if args.no_cpu_baseline else batched_cpu_baseline(probs, tol)
    out = {
        "workload": f"ordinal_batch_B{B}_N32-4096", "B": B, "tolerance": tol,
        "config": "N log-uniform [32,4096], D in {1,2,4,8}, J in 2..7, kernel in {EQ, Matern12, EQ.periodic(0.5)}, "
                  "l ~ LogU[0.3,3], s ~ LogU[0.5,2], noise std sqrt(0.4), seed 2",
        "value": B / (batched_ms / 1e3), "unit": UNIT, "ms_per_batch": batched_ms,
        "e2e": {"value": B / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(Xp.nbytes + yp.nbytes + 4 * theta.numel()),
                "d2h_bytes_per_step": int(4 * (B + theta.numel()))},
        "newton_iterations": {"mean": float(iters.mean()), "max": int(iters.max()),
                              "at_maxiter": int((iters >= 100).sum()),
                              "at_maxiter_problems": [
                                  {"index": int(k), "N": int(probs[k].X.shape[0]), "D": int(probs[k].X.shape[1]),
                                   "J": int(probs[k].J), "kernel": probs[k].kernel}
                                  for k in np.nonzero(iters >= 100)[0][:8]]},
        "algorithmic_tflop": float((Ns ** 3 / 3).sum() * (iters.mean() + 3) / 1e12),
        "gpu_launches_per_batch": launches_per_solve(int(iters.max()), *kernel_groups(probs)),
        "data_generation_s": gen_s,
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if args.no_plain:
        return out
    # plain path: one single-GP value_and_grad per problem (handles and graphs prepared first)
    lib = N.load()
    handles, Xs, ys, ths = [], [], [], []
    for b, q in enumerate(probs):
        h = C.c_void_p()
        N.check(lib.pgb_gp_create(batch.descs[b], C.byref(h)), "pgb_gp_create")
        handles.append(h)
        Xs.append(torch.from_numpy(q.X).to(dev))
        ys.append(torch.from_numpy(q.y).to(dev))
        ths.append(td[int(batch.theta_off[b]):int(batch.theta_off[b + 1])].contiguous())
    vals = torch.empty(B, dtype=torch.float32, device=dev)
    grads = torch.empty(int(batch.theta_off[-1]), dtype=torch.float32, device=dev)
    sh = stream.cuda_stream

    def plain():
        for b in range(B):
            N.check(lib.pgb_value_and_grad(handles[b], Xs[b].data_ptr(), ys[b].data_ptr(), ths[b].data_ptr(),
                                           vals[b:].data_ptr(), grads[int(batch.theta_off[b]):].data_ptr(), sh),
                    "pgb_value_and_grad")

    plain()
    torch.cuda.synchronize()
    same = bool(torch.equal(vals, batch.value_and_grad_flat(td)[0]))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plain()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    for h in handles:
        lib.pgb_gp_destroy(h)
    out["plain"] = {"value": B / (plain_ms / 1e3), "unit": UNIT, "ms_per_batch": plain_ms,
                    "what": "one pgb_value_and_grad (CUDA graph) per problem, same kernels, no host sync between"}
    out["batched_over_plain"] = plain_ms / batched_ms
    out["results_identical_to_plain"] = same
    return out


def batched_cpu_baseline(probs, tol, nsample=12):
    """The oracle (the reference algorithm in NumPy/SciPy, float32, all host
    threads) on problems at evenly spaced quantiles of N, extrapolated to the
    whole batch with a power law t(N) fitted in log-log."""
    from oracle import laplace as L

    order = np.argsort([q.N for q in probs])
    pick = [int(order[int(round(k))]) for k in np.linspace(0, len(probs) - 1, nsample)]
    Ns, ts = [], []
    t_all = time.perf_counter()
    for b in pick:
        q = probs[b]
        op = L.Problem(q.X, q.y, q.kernel, "probit", 1, q.period, q.J)
        t0 = time.perf_counter()
        L.value_and_grad(op, q.theta().astype(np.float32), tol=tol, dtype=np.float32)
        ts.append(time.perf_counter() - t0)
        Ns.append(q.N)
    coef = np.polyfit(np.log(Ns), np.log(ts), 1)
    total = float(np.exp(np.polyval(coef, np.log([q.N for q in probs]))).sum())
    return {"value": len(probs) / total, "unit": UNIT, "cores": len(os.sched_getaffinity(0)), "kind": "port",
            "sample": f"{nsample} problems at N quantiles {sorted(Ns)} timed with the NumPy/SciPy restatement of "
                      f"the reference algorithm (float32, OpenBLAS on all host threads) in "
                      f"{time.perf_counter() - t_all:.1f} s; extrapolated to all {len(probs)} problems with "
                      f"t ~ N^{coef[0]:.2f}"}


def run_hyperopt(args, dev):
    """The hyperparameter-optimisation workload: B ordinal GPs (N uniform in
    [256, 2048], D = 3, J = 5, Matern12) each fitted by lockstep L-BFGS on
    (log l, log s, log sigma, interior cutpoints); every evaluation round is
    one batched evidence + gradient call."""
    import ctypes as C

    import torch

    import probit_gb300 as pg
    from probit_gb300 import _native as N
    from probit_gb300 import workloads as Wk
    from probit_gb300.optimize import LogParams, batch_objective, minimize_lockstep

    B = args.hyperopt
    probs = Wk.hyperopt_c3(B=B, device=dev)
    tol = args.batch_tol
    gps = [pg.LaplaceGP((q.X, q.y), q.prior(), pg.log_probit_likelihood, tolerance=tol) for q in probs]
    params = [q.params() for q in probs]
    batch = pg.LaplaceBatch(gps, params)
    lp = LogParams(nl=1, J=5)
    rng = np.random.default_rng(30)
    th0 = np.stack([np.asarray(q.theta(), np.float64) for q in probs])
    th0[:, 4:8] *= rng.uniform(0.7, 1.3, size=(B, 1))        # interior cutpoints scaled, still ordered
    u0 = lp.from_theta(th0)
    u0[:, :3] += rng.normal(0.0, 0.5, size=(B, 3))          # log l, log s, log sigma away from the truth
    fg_batch = batch_objective(batch, lp)
    solved = [0]

    def fg(U, mask=None):
        solved[0] += B if mask is None else int(np.count_nonzero(mask))
        return fg_batch(U, mask)

    for _ in range(max(3, args.warmup)):
        fg(u0)
    torch.cuda.synchronize()
    f0, _ = fg(u0)
    solved[0] = 0
    t0 = time.perf_counter()
    res = minimize_lockstep(fg, u0, maxiter=args.hyperopt_steps)
    wall = time.perf_counter() - t0
    evals = res.evaluations
    batch.set_enabled(None)
    st = batch.status()
    out = {
        "workload": f"hyperopt_B{B}_N256-2048_D3_J5_matern12", "B": B, "lbfgs_steps": args.hyperopt_steps,
        "tolerance": tol, "evaluation_rounds": evals, "problem_evaluations": solved[0], "wall_s": wall,
        "value": solved[0] / wall, "unit": UNIT,
        "what": "end to end: host L-BFGS (vectorised over problems) + one batched value_and_grad per round "
                "over the problems whose line search runs (the others are masked off), theta up and values + "
                "gradients down every round; value = problem evaluations / wall time",
        "objective_mean": {"start": float(np.mean(f0)), "end": float(np.mean(res.f))},
        "accepted_steps_mean": float(res.iterations.mean()),
        "problems_failed": int(sum(1 for x in st if x[0] != 0)),
    }
    # plain path: one single-GP value_and_grad per problem for one round at the final point
    theta = torch.from_numpy(lp.to_theta(res.x).astype(np.float32).reshape(-1)).to(dev)
    lib = N.load()
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    handles, Xs, ys = [], [], []
    for b, q in enumerate(probs):
        h = C.c_void_p()
        N.check(lib.pgb_gp_create(batch.descs[b], C.byref(h)), "pgb_gp_create")
        handles.append(h)
        Xs.append(torch.from_numpy(q.X).to(dev))
        ys.append(torch.from_numpy(q.y).to(dev))
    vals = torch.empty(B, dtype=torch.float32, device=dev)
    grads = torch.empty(theta.numel(), dtype=torch.float32, device=dev)
    off = batch.theta_off

    def plain():
        for b in range(B):
            N.check(lib.pgb_value_and_grad(handles[b], Xs[b].data_ptr(), ys[b].data_ptr(),
                                           theta[int(off[b]):].data_ptr(), vals[b:].data_ptr(),
                                           grads[int(off[b]):].data_ptr(), sh), "pgb_value_and_grad")

    plain()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plain()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    e0.record(stream)
    batch.value_and_grad_flat(theta)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1)
    for h in handles:
        lib.pgb_gp_destroy(h)
    out["batched_round_ms"] = batched_ms
    out["plain"] = {"value": B / (plain_ms / 1e3), "unit": UNIT, "round_ms": plain_ms,
                    "what": "one pgb_value_and_grad per problem per evaluation round (device time)"}
    out["batched_over_plain"] = plain_ms / batched_ms
    if not args.no_cpu_baseline:
        cpu = batched_cpu_baseline(probs, tol, nsample=8)
        out["cpu_baseline"] = cpu
        out["e2e_over_cpu"] = out["value"] / cpu["value"]
    return out


def run_serving(args, dev):
    """The serving workload: Poisson arrivals of fit / evidence+gradient /
    predict requests against a pool of 256 resident GP models (generated as
    the batched workload, N 32..8192), served with continuous batching; p50 /
    p99 latency (arrival to result on the host) and throughput."""
    from probit_gb300 import serving as S
    from probit_gb300 import workloads as Wk

    out = {"workers": args.serve_workers, "pool": 256, "max_large": args.serve_max_large,
           "large_blocks": args.serve_large_blocks, "small_blocks": args.serve_small_blocks}
    for tag, rate, dur, seed in (("offered_2000_per_s", 2000.0, args.serve_seconds, 4),
                                 ("offered_150_per_s", 150.0, max(5.0, args.serve_seconds), 5)):
        probs, reqs = Wk.serving_c4(rate=rate, duration=dur, pool=256, seed=seed, device=dev)
        gc.collect()   # the previous run's objects are not collected during this one
        srv = S.Server(workers=args.serve_workers, max_large=args.serve_max_large,
                       large_blocks=args.serve_large_blocks, small_blocks=args.serve_small_blocks, warm_large=True)
        try:
            t0 = time.perf_counter()
            srv.replay([S.Request(0.0, "fit", k, p) for k, p in enumerate(probs)], realtime=False)
            srv.wait_idle()   # warm-ups of the fitted models finish before the arrivals start
            prefit = time.perf_counter() - t0
            gc.collect()
            gc.freeze()    # objects alive now are never scanned by a collection during the replay
            try:
                done = srv.replay(reqs, realtime=True)
            finally:
                gc.unfreeze()
            summ = S.latency_summary(done)
            compact = {"p50_ms": summ["all"]["p50_ms"], "p99_ms": summ["all"]["p99_ms"],
                       "small_p50_ms": summ["n<=2048"]["p50_ms"], "small_p99_ms": summ["n<=2048"]["p99_ms"],
                       "req_s": summ["throughput_req_s"], "requests": len(reqs), "errors": summ["errors"],
                       "window_s": dur}
        finally:
            srv.close()
        out[tag] = compact
    return out


def run_c0(args, dev):
    """Config 0: the reference's ordinal classification example scaled up
    (N = 512, D = 2, J = 3, Matern12, 1,000-point grid), at the reference's
    default tolerance 1e-5.  One step = approximate_posterior + value_and_grad
    + predict, through the public LaplaceGP API with host inputs (e2e) and
    through the C-ABI with resident inputs (device-timed)."""
    import ctypes as C

    import torch

    import probit_gb300 as pg
    from oracle import laplace as L
    from probit_gb300 import _native as N
    from probit_gb300 import workloads as Wk

    tol = 1e-5
    p = Wk.ordinal_c0()
    M = p.Xtest.shape[0]
    lib = N.load()
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    th = p.theta().astype(np.float32)
    Xd, yd, td = (torch.from_numpy(x).to(dev) for x in (p.X, p.y, th))
    Xs = torch.from_numpy(p.Xtest).to(dev)
    desc = N.Desc(p.N, p.D, N.KERNEL_MATERN12, 1, 0.5, N.LIK_PROBIT, p.J, tol, 100, 0)
    h = C.c_void_p()
    N.check(lib.pgb_gp_create(desc, C.byref(h)), "pgb_gp_create")
    a, Wv = torch.empty(p.N, device=dev), torch.empty(p.N, device=dev)
    out = torch.empty(th.size + 1, device=dev)
    mean, var = torch.empty(M, device=dev), torch.empty(M, device=dev)

    def step():
        N.check(lib.pgb_approximate_posterior(h, Xd.data_ptr(), yd.data_ptr(), td.data_ptr(), a.data_ptr(),
                                              Wv.data_ptr(), sh), "posterior")
        N.check(lib.pgb_value_and_grad(h, Xd.data_ptr(), yd.data_ptr(), td.data_ptr(), out.data_ptr(),
                                       out[1:].data_ptr(), sh), "value_and_grad")
        N.check(lib.pgb_predict(h, Xd.data_ptr(), td.data_ptr(), a.data_ptr(), Wv.data_ptr(), Xs.data_ptr(), M,
                                mean.data_ptr(), var.data_ptr(), 1, sh), "predict")

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    st = N.Status()
    lib.pgb_gp_status(h, C.byref(st), sh)
    reps = max(3, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    dev_ms = e0.elapsed_time(e1) / reps
    v_gpu = float(out[0].item())
    lib.pgb_gp_destroy(h)
    # end to end through LaplaceGP with host (numpy) inputs and outputs
    gp = pg.LaplaceGP((p.X, p.y), p.prior(), pg.log_probit_likelihood, tolerance=tol, array_type="numpy")
    params = p.params()
    for _ in range(2):
        aa, WW = gp.approximate_posterior(params)
        gp.value_and_grad()(params)
        gp.predict(p.Xtest, params, aa, WW)
    t0 = time.perf_counter()
    for _ in range(reps):
        aa, WW = gp.approximate_posterior(params)
        vv, gg = gp.value_and_grad()(params)
        mm, ss = gp.predict(p.Xtest, params, aa, WW)
    e2e_ms = 1e3 * (time.perf_counter() - t0) / reps
    out_d = {"workload": "ordinal_c0_N512_D2_J3_matern12_M1000", "tolerance": tol,
             "newton_iterations": int(st.iterations), "device_ms_per_step": dev_ms, "e2e_ms_per_step": e2e_ms,
             "value": 1e3 / dev_ms, "unit": "steps/s (posterior + evidence+grad + predict)"}
    if not args.no_cpu_baseline:
        op = L.Problem(p.X.astype(np.float64), p.y, "matern12", "probit", 1, 0.5, 3)
        t0 = time.perf_counter()
        a32, it32 = L.newton_weight(op, th, tol=tol, dtype=np.float32)
        W32, _ = L.precision(op, th, a32, dtype=np.float32)
        v32, _, _, _ = L.value_and_grad(op, th, tol=tol, dtype=np.float32)
        L.predict(op, th, p.Xtest, a32, W32, dtype=np.float32)
        cpu_s = time.perf_counter() - t0
        a64, it64 = L.newton_weight(op, p.theta(), tol=tol)
        v64 = L.objective_bform(op, p.theta(), a64)
        out_d["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "steps/s", "cores": len(os.sched_getaffinity(0)),
                                 "kind": "port", "newton_iterations": int(it32),
                                 "sample": "1 step (weight, precision, value_and_grad, predict) of the NumPy/SciPy "
                                           "restatement in float32 (LU Newton; at tolerance 1e-5 it stalls at "
                                           "its rounding floor and runs to maxiter 100)"}
        out_d["accuracy"] = {"rel_err_vs_float64": abs(v_gpu - float(v64)) / abs(float(v64)),
                             "rel_err_vs_float32_port": abs(v_gpu - float(v32)) / abs(float(v32)),
                             "float64_newton_iterations": int(it64)}
    return out_d


def run_sharded(args, dev, ws, rank):
    """Config 2 sharded over the ranks: each rank evaluates its
    longest-processing-time share (by N^3) of the 1,024 problems in one
    LaplaceBatch on its GPU; values and gradients are gathered as host
    objects.  value = problems / (max over ranks of the wall time per round)."""
    import torch

    import probit_gb300 as pg
    from probit_gb300 import workloads as Wk
    from probit_gb300.shard import run_sharded_rounds

    probs = Wk.batched_c2(B=args.batch, device=dev)
    gps = [pg.LaplaceGP((q.X, q.y), q.prior(), pg.log_probit_likelihood, tolerance=args.batch_tol) for q in probs]
    params = [q.params() for q in probs]
    res = run_sharded_rounds(gps, params, rounds=max(1, min(args.steps, 5)), warmup=max(3, args.warmup),
                             rank=rank, world=ws, sync=torch.cuda.synchronize)
    return {"workload": f"ordinal_batch_B{args.batch}_N32-4096 sharded by N^3 (LPT)", "ranks": res["ranks"],
            "value": res["value"], "unit": UNIT, "rounds": res["rounds"], "max_s_per_round": res["max_s"] / res["rounds"],
            "local_problems_rank0": res["local_problems"],
            "what": "end to end per round: every rank's LaplaceBatch evaluation of its share plus the host gather "
                    "of all values and gradients; no device collective"}


def summary_of(line):
    """The few figures each section is judged on, kept short so they stay in
    the tail of the output line."""
    out = {}
    acc = line.get("accuracy") or {}
    if "rel_err" in acc:
        out["c1_rel_err"] = acc["rel_err"]
        if acc.get("predict"):
            out["c1_predict_err"] = [acc["predict"]["mean_err_of_max"], acc["predict"]["var_err_of_s"]]
    if line.get("predict"):
        out["c1_predict_ms"] = line["predict"]["ms"]
    c0 = line.get("c0")
    if c0:
        out["c0"] = {"ms": c0["device_ms_per_step"], "e2e_ms": c0["e2e_ms_per_step"], "iters": c0["newton_iterations"]}
        if c0.get("accuracy"):
            out["c0"]["rel_err"] = c0["accuracy"]["rel_err_vs_float64"]
        if c0.get("cpu_baseline"):
            out["c0"]["cpu_steps_s"] = c0["cpu_baseline"]["value"]
    b = line.get("batched")
    if b:
        out["c2"] = {"value": b["value"], "e2e": b["e2e"]["value"]}
        if "plain" in b:
            out["c2"].update(plain=b["plain"]["value"], batched_over_plain=b["batched_over_plain"],
                             identical=b["results_identical_to_plain"])
        if "cpu_baseline" in b:
            out["c2"]["cpu"] = b["cpu_baseline"]["value"]
    ho = line.get("hyperopt")
    if ho:
        out["c3"] = {"value": ho["value"], "rounds": ho["evaluation_rounds"],
                     "batched_over_plain": ho.get("batched_over_plain"), "e2e_over_cpu": ho.get("e2e_over_cpu")}
    sv = line.get("served")
    if sv:
        out["c4"] = {k: v for k, v in sv.items() if isinstance(v, dict)}
    if line.get("sharded_c2"):
        out["sharded_c2"] = {"ranks": line["sharded_c2"]["ranks"], "value": line["sharded_c2"]["value"]}
    return out


def kernel_groups(probs):
    """(gradient-trace launches, Gram-matvec launches) of a batch: one per
    (feature width class, periodic) and per (kernel, feature width class)."""
    def dm(q):
        F = 2 * q.D if q.kernel == "eq_periodic" else q.D
        Dp = (F + 3) // 4 * 4
        return 4 if Dp <= 4 else (8 if Dp <= 8 else 16)
    trace = {(dm(q), q.kernel == "eq_periodic") for q in probs}
    mv = {(dm(q), q.kernel) for q in probs}
    return len(trace), len(mv)


# ---------------------------------------------------------------- GB300 arm
def run_gb300(args, ws, rank, local):
    import ctypes as C

    import torch

    import __graft_entry__ as ge

    ge.build()
    import probit_gb300 as pg
    from probit_gb300 import _native as N
    from probit_gb300 import workloads as Wk

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = N.load()
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    p = Wk.regression_c1(N=args.n, M=args.predict_m)
    n, D = p.N, p.D
    theta_np = p.theta().astype(np.float32)
    P = theta_np.size
    Xd = torch.from_numpy(p.X).to(dev)
    yd = torch.from_numpy(p.y).to(dev)
    td = torch.from_numpy(theta_np).to(dev)
    desc = N.Desc(n, D, N.KERNEL_EQ, 4, 1.0, N.LIK_GAUSSIAN, 0, TOL, 100, 0)
    h = C.c_void_p()
    N.check(lib.pgb_gp_create(desc, C.byref(h)), "pgb_gp_create")
    out = torch.empty(1 + P, dtype=torch.float32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > L2

    def step():
        N.check(lib.pgb_value_and_grad(h, Xd.data_ptr(), yd.data_ptr(), td.data_ptr(), out.data_ptr(),
                                       out[1:].data_ptr(), sh), "pgb_value_and_grad")

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    st = N.Status()
    lib.pgb_gp_status(h, C.byref(st), sh)
    iters = st.iterations
    # ---- device-timed region (inputs resident in HBM; L2 flushed between steps)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = sum(step_ms)
    t_ms = max_over_ranks(t_ms, ws)
    value = ws * args.steps / (t_ms / 1e3)
    clocks = clk.summary()

    # ---- dominant kernel live: the tile-DAG factorisation of B (no RHS)
    fe = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
    for a, b in fe:
        flush.zero_()
        a.record(stream)
        N.check(lib.pgb_factor(h, sh), "pgb_factor")
        b.record(stream)
    torch.cuda.synchronize()
    f_ms = statistics.median(a.elapsed_time(b) for a, b in fe)
    flops = n ** 3 / 3.0
    pk, pk_kind = peaks()
    achieved_tf = flops / (f_ms / 1e3) / 1e12
    peak_tf = pk["bf16_tflops"]

    # ---- end to end through the public API, host buffers, H2D + D2H each step
    Xh = torch.from_numpy(p.X).pin_memory()
    yh = torch.from_numpy(p.y).pin_memory()
    gp = pg.LaplaceGP((Xh, yh), p.prior(), pg.log_gaussian_likelihood, tolerance=TOL, array_type="numpy")
    params = p.params()
    vg = gp.value_and_grad()
    for _ in range(2):
        gp.data = (Xh, yh)
        vg(params)
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gp.data = (Xh, yh)          # inputs re-uploaded from pinned host memory
        value_e2e, grads = vg(params)   # value + gradient read back to the host
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    e2e = ws * args.steps / e2e_s
    h2d = p.X.nbytes + p.y.nbytes + 4 * P
    d2h = 4 * (1 + P)

    # ---- predict at M test points (reported beside the headline)
    pred = None
    pred_mv = (None, None)
    if args.predict_m > 0 and rank == 0:
        Xs = torch.from_numpy(p.Xtest).to(dev)
        a = torch.empty(n, device=dev)
        Wv = torch.empty(n, device=dev)
        N.check(lib.pgb_approximate_posterior(h, Xd.data_ptr(), yd.data_ptr(), td.data_ptr(), a.data_ptr(),
                                              Wv.data_ptr(), sh), "posterior")
        mean = torch.empty(args.predict_m, device=dev)
        var = torch.empty_like(mean)
        times = []
        for _ in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            N.check(lib.pgb_predict(h, Xd.data_ptr(), td.data_ptr(), a.data_ptr(), Wv.data_ptr(), Xs.data_ptr(),
                                    args.predict_m, mean.data_ptr(), var.data_ptr(), 1, sh), "pgb_predict")
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        pf = float(n) * n * args.predict_m
        pred = {"M": args.predict_m, "ms": min(times), "tflops_algorithmic": pf / (min(times) / 1e3) / 1e12}
        pred_mv = (mean.cpu().numpy(), var.cpu().numpy())

    # the same solve at the reference's default tolerance 1e-5 (once, untimed
    # loop): float32 stalls above it, so the Newton loop runs to maxiter on
    # reused factors
    ref_tol = None
    if rank == 0:
        desc5 = N.Desc(n, D, N.KERNEL_EQ, 4, 1.0, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
        h5 = C.c_void_p()
        N.check(lib.pgb_gp_create(desc5, C.byref(h5)), "pgb_gp_create")
        o5 = torch.empty(1 + P, dtype=torch.float32, device=dev)
        for rep in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            N.check(lib.pgb_value_and_grad(h5, Xd.data_ptr(), yd.data_ptr(), td.data_ptr(), o5.data_ptr(),
                                           o5[1:].data_ptr(), sh), "pgb_value_and_grad")
            e1.record(stream)
            torch.cuda.synchronize()
        st5 = N.Status()
        lib.pgb_gp_status(h5, C.byref(st5), sh)
        ref_tol = {"tolerance": 1e-5, "newton_iterations": int(st5.iterations), "ms": e0.elapsed_time(e1),
                   "value_diff_vs_headline": float(o5[0].item()) - float(out[0].item())}
        lib.pgb_gp_destroy(h5)

    launches_per_step = launches_per_solve(iters, factor_steps=1)   # Gaussian: only the first step factors
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": config_name(n), "N": n, "D": D, "kernel": "EQ ARD (0.5,1,1.5,2)", "likelihood":
                   "gaussian sigma=0.2", "tolerance": TOL, "newton_iterations": iters,
                   "parallelism": "replicas" if ws > 1 else "single", "l2": "256 MB buffer written between steps",
                   "at_reference_tolerance": ref_tol},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"kernel": "dag_factor_kernel (Cholesky of B, N^3/3 flop)", "bound": "tensor",
                     "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s", "frac": achieved_tf / peak_tf,
                     "peak_kind": f"{pk_kind} bf16 dense", "launch_ms": f_ms,
                     "traffic": FACTOR_TRAFFIC_N8192 if n == 8192 else None,
                     "frac_of_3xtf32_nominal": achieved_tf / (TF32_NOMINAL_TFLOPS / 3.0)},
        "clocks": clocks,
        "gpu_launches": launches_per_step * args.steps,
        "predict": pred,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    if rank == 0 and ws == 1 and not args.no_accuracy:
        line["accuracy"] = accuracy_check(p, float(out[0].item()), *pred_mv)
    lib.pgb_gp_destroy(h)
    del flush
    if rank == 0 and ws == 1 and not args.no_c0:
        line["c0"] = run_c0(args, dev)
    if rank == 0 and ws == 1 and args.batch > 0:
        line["batched"] = run_batched(args, dev)
        b = line["batched"]
        line["sharded_c2"] = {"ranks": 1, "value": b["e2e"]["value"], "unit": UNIT,
                              "what": "one rank: the whole batch in one LaplaceBatch, end to end"}
    if ws > 1 and args.batch > 0:
        line["sharded_c2"] = run_sharded(args, dev, ws, rank)
    if rank == 0 and ws == 1 and args.hyperopt > 0:
        line["hyperopt"] = run_hyperopt(args, dev)
    if rank == 0 and ws == 1 and args.serve_seconds > 0:
        line["served"] = run_serving(args, dev)
    if rank == 0:
        line["summary"] = summary_of(line)   # last: the tail of the line
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gb300(args, ws, rank, local)
    if ws > 1 and args.impl == "gb300":
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
