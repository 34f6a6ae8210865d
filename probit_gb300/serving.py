"""Serving: fit / evidence+gradient / predict requests with continuous batching.

A :class:`Server` takes requests as they arrive and runs them concurrently on
one GPU:

* every fitted GP (a *model*) stays resident in HBM as a library handle
  holding its factor L of B, W, a and the features; a predict request reuses
  that factor (``pgb_predict`` with ``reuse_factor``), so it costs one
  cross-kernel solve and no refactorisation;
* requests are admitted by HBM footprint: a request runs only when its
  workspace (and, for a fit, its resident model) fits in the memory budget;
  idle models are evicted least-recently-used when room is needed;
* admitted requests run on a pool of worker threads, each driving its own
  CUDA stream, so the kernels of different requests overlap on the device
  (the tile-DAG launches of small problems use a few SMs each); requests of
  small problems (n <= ``small_n``) go to higher-priority streams and are
  taken first, some workers take only them, at most ``max_large`` large
  problems run at a time and their launches are capped at ``large_blocks``
  persistent blocks, so the SMs left over always serve small requests (a
  large request's latency then absorbs the overload, a small one's does
  not); small problems' launches are capped too (``small_blocks``), so
  that several small requests share the remaining SMs at once instead of
  queueing behind one another's persistent blocks (a persistent block holds
  its SM until its launch ends); the streams need as many hardware work
  queues (``CUDA_DEVICE_MAX_CONNECTIONS``, set before CUDA is initialised),
  or requests on streams that share a queue wait for each other;
* a model is used by one request at a time (a handle is not thread-safe);
  other requests for it wait in the queue.

Results are what the same call gives alone: every kernel's arithmetic for a
problem is independent of what else runs on the GPU.

The request semantics follow the reference's methods: a fit is
``approximate_posterior`` (``approximators.py:204-210``), an evidence+gradient
request is ``value_and_grad`` (``approximators.py:132-134``), a predict
request is ``predict`` (``approximators.py:154-180``) at the model's resident
posterior.
"""

from __future__ import annotations

import ctypes as C
import heapq
import itertools
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N

_KINDS = {"eq": N.KERNEL_EQ, "matern12": N.KERNEL_MATERN12, "eq_periodic": N.KERNEL_EQ_PERIODIC}


def handle_bytes(n, d, kind, grad=True, m=0):
    """HBM a handle of n points needs (workspace + resident factor), plus the
    predict workspace for m test points."""
    npad = -(-n // 128) * 128
    nt = npad // 128
    F = 2 * d if kind == "eq_periodic" else d
    Fp = -(-F // 4) * 4
    mat = 4 * npad * npad
    vec = 4 * npad * (22 + Fp)
    # L in fp32 and as its TF32 hi/lo split, the same for the diagonal
    # inverses and the Newton right-hand-side row tile, vectors, partial sums,
    # tile flags
    b = 3 * mat + 3 * 4 * nt * 128 * 128 + 3 * 4 * 128 * npad + vec + 8 * npad * 80         + 4 * ((2 * nt + 1) * nt + 2 * nt) + 16 * nt * nt + 4096
    if grad:
        b += 3 * mat          # split L^-T and B^-1
    if m > 0:
        mpad = -(-m // 128) * 128
        b += 4 * mpad * (2 * npad + nt + Fp + d + 2) + 4 * (nt + mpad // 128) * nt
    return b


def work_queue_setting(workers, current, cuda_initialized):
    """(value to set CUDA_DEVICE_MAX_CONNECTIONS to or None, warning or None)
    for a server of `workers` workers, two streams each (at most 32 hardware
    queues exist).  `current` is the variable's value (None: unset, which
    means 8).  Before the CUDA context exists an unset variable is set;
    afterwards a count below the streams only draws a warning."""
    want = max(8, min(32, 2 * workers))
    try:
        have = int(current) if current is not None else None
    except ValueError:
        have = None
    if not cuda_initialized:
        return (str(want) if current is None else None), None
    if (have if have is not None else 8) < want:
        return None, (f"CUDA_DEVICE_MAX_CONNECTIONS={current or 8} < {want} streams: requests on streams that "
                      "share a hardware queue are serialised; set it before CUDA is initialised")
    return None, None


@dataclass
class Problem:
    """The data and hyperparameters of one served GP (host arrays)."""

    X: np.ndarray            # (n, d) float32
    y: np.ndarray            # (n,) int32 labels (ordinal probit) or float32 targets (Gaussian)
    kind: str                # "eq" | "matern12" | "eq_periodic"
    theta: np.ndarray        # flat theta: l, s, sigma, cutpoints (J + 1, infinite ends)
    nl: int = 1
    J: int = 0               # 0: Gaussian likelihood
    period: float = 0.5
    tolerance: float = 1e-3
    maxiter: int = 100

    @property
    def n(self):
        return self.X.shape[0]

    @property
    def d(self):
        return self.X.shape[1]

    def desc(self):
        lik = N.LIK_GAUSSIAN if self.J == 0 else N.LIK_PROBIT
        return N.Desc(self.n, self.d, _KINDS[self.kind], self.nl, self.period, lik, self.J, self.tolerance,
                      self.maxiter, 0)


@dataclass(order=True)
class Request:
    sort_key: tuple = field(init=False, repr=False)
    arrival: float                     # seconds since the start of the run
    kind: str = field(compare=False)   # "fit" | "vg" | "predict"
    model: int = field(compare=False)  # model id (fit: the id it creates)
    problem: Problem = field(compare=False, default=None)
    Xs: np.ndarray = field(compare=False, default=None)    # predict: (m, d) float32
    theta: np.ndarray = field(compare=False, default=None)  # vg: hyperparameters to evaluate
    # filled in by the server
    start: float = field(compare=False, default=None)
    done: float = field(compare=False, default=None)
    result: tuple = field(compare=False, default=None)
    error: str = field(compare=False, default=None)

    def __post_init__(self):
        self.sort_key = (self.arrival,)

    @property
    def n(self):
        return self.problem.n

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


class _Model:
    def __init__(self, mid, problem):
        self.id = mid
        self.problem = problem
        self.h = None          # handle of the fit and its predicts (resident posterior)
        self.hvg = None        # handle of evidence + gradient requests (own factor, L^-T, B^-1)
        self.cap_m = 0         # predict rows the fit handle has workspace for
        self.bytes = 0         # HBM held by the handles (as accounted)
        self.busy = False
        self.fitted = False
        self.last_used = 0.0
        self.dev = {}          # device tensors: X, y, theta, a, W

    def footprint(self, fit, vg, cap_m):
        p = self.problem
        b = handle_bytes(p.n, p.d, p.kind, grad=False, m=cap_m) if fit else 0
        if vg:
            b += handle_bytes(p.n, p.d, p.kind, grad=True)
        return b


class Server:
    """Continuous-batching request server on the current CUDA device."""

    def __init__(self, workers=12, mem_budget=None, small_n=2048, large_blocks=24, small_only=4, warm_small=True,
                 warm_rows=4096, max_large=5, warm_large=False, small_blocks=32, switch_interval=2e-4):
        import os
        import sys
        import warnings

        import torch

        # Every worker drives two streams.  The CUDA context multiplexes streams
        # onto a fixed number of hardware work queues (CUDA_DEVICE_MAX_CONNECTIONS,
        # 8 unless set, read when the context is created); streams that share a
        # queue are ordered, so a small request's kernel could wait behind a
        # large request's launch.  Before the context exists the server asks
        # for enough queues; after, it can only warn.
        setting, warning = work_queue_setting(workers, os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                                              torch.cuda.is_initialized())
        if setting is not None:
            os.environ["CUDA_DEVICE_MAX_CONNECTIONS"] = setting
        if warning is not None:
            warnings.warn(warning, RuntimeWarning, stacklevel=2)

        # the worker threads, the submitting thread and the caller share one
        # interpreter lock; CPython hands it over every 5 ms by default, which
        # puts multiples of 5 ms into the latency of a request whose thread
        # waits for it.  The server sets a shorter interval while it runs
        # (process wide; close() restores the previous one; None leaves it).
        self._old_switch = sys.getswitchinterval()
        if switch_interval is not None:
            sys.setswitchinterval(switch_interval)

        self.torch = torch
        self.lib = N.load()
        self.device = torch.device("cuda", torch.cuda.current_device())
        free, _ = torch.cuda.mem_get_info(self.device)
        self.budget = int(mem_budget if mem_budget is not None else 0.6 * free)
        self.used = 0
        self.small_n = small_n
        self.large_blocks = large_blocks   # SM share of the launches of a problem with n > small_n
        self.small_blocks = small_blocks   # the same for n <= small_n (0: one block per SM)
        self.max_large = max_large         # large requests running at once (0: no limit)
        self.large_running = 0
        # after the first fit of a small model, its evidence + gradient handle is
        # created and its graph captured (one evaluation at the fitted
        # hyperparameters) and its predict workspace sized for `warm_rows`
        # test points (one prediction) before the model is released, so no
        # request pays a first-use graph build or workspace allocation
        self.warm_small = warm_small
        # the same warm-up for large models (their first evidence + gradient
        # request otherwise grows the memory pool and captures a graph while
        # other requests run)
        self.warm_large = warm_large
        self.warm_rows = int(warm_rows)
        self.warm_errors = []          # warm-ups that failed (the first request then builds instead)
        self.busy_workers = 0
        self.models: dict[int, _Model] = {}
        self.evicted = set()
        self.lock = threading.Condition()
        self.heaps = ([], [])         # small / large requests: (arrival, seq, request)
        self.seq = itertools.count()
        self.stop = False
        self.t0 = time.perf_counter()
        self.evictions = 0
        lo, hi = torch.cuda.Stream.priority_range()
        small_only = min(small_only, max(0, workers - 2))   # at least two workers take large requests
        self.workers = []
        for w in range(workers):
            # roles: the first `small_only` workers take only small requests (so a
            # small request never waits behind large ones for a worker), then half
            # the rest prefer small requests; both run on high-priority streams
            if w < small_only:
                role = "small"
            elif w < small_only + (workers - small_only + 1) // 2:
                role = "small_first"
            else:
                role = "any"
            # small requests on a high-priority stream, large ones on a low-priority
            # one: blocks of small requests' launches are scheduled first
            streams = (torch.cuda.Stream(device=self.device, priority=hi),
                       torch.cuda.Stream(device=self.device, priority=lo))
            t = threading.Thread(target=self._worker, args=(streams, role), daemon=True)
            self.workers.append(t)
            t.start()

    # -- clock -----------------------------------------------------------------
    def now(self):
        return time.perf_counter() - self.t0

    # -- submission -------------------------------------------------------------
    def submit(self, req: Request):
        if req.kind not in ("fit", "vg", "predict"):
            raise ValueError(f"unknown request kind {req.kind!r}")
        if req.kind == "predict":
            Xs = np.asarray(req.Xs)
            if Xs.ndim != 2 or Xs.shape[0] < 1 or Xs.shape[1] != req.problem.d:
                raise ValueError(f"predict request: Xs must be (m >= 1, {req.problem.d}), got {Xs.shape}")
        if req.kind == "vg" and req.theta is not None:
            want = self.lib.pgb_theta_size(req.problem.desc())
            if np.asarray(req.theta).size != want:
                raise ValueError(f"vg request: theta must have {want} entries, got {np.asarray(req.theta).size}")
        with self.lock:
            cls = 0 if req.n <= self.small_n else 1
            heapq.heappush(self.heaps[cls], (req.arrival, next(self.seq), req))
            self.lock.notify_all()

    def _pending(self):
        return bool(self.heaps[0] or self.heaps[1])

    def close(self):
        import sys

        with self.lock:
            self.stop = True
            self.lock.notify_all()
        for t in self.workers:
            t.join()
        for m in list(self.models.values()):
            self._destroy(m)
        sys.setswitchinterval(self._old_switch)

    # -- admission --------------------------------------------------------------
    def _plan(self, req, m):
        """(handles after the request: fit, vg, cap_m) for `req` on model `m`."""
        fit, vg, cap = m.h is not None, m.hvg is not None, m.cap_m
        if req.kind == "fit":
            fit = True
        elif req.kind == "vg":
            vg = True
        else:
            cap = max(cap, -(-req.Xs.shape[0] // 128) * 128)
        return fit, vg, cap

    def _runnable(self, req):
        """Called with the lock held: can `req` start now (model state, memory)?"""
        m = self.models.get(req.model)
        if req.kind == "predict" and (m is None or not m.fitted):
            return False
        if m is not None and m.busy:
            return False
        probe = m if m is not None else _Model(req.model, req.problem)
        need = probe.footprint(*self._plan(req, probe)) - probe.bytes
        if self.used + need > self.budget:
            self._evict(self.used + need - self.budget, keep=req.model)
            if self.used + need > self.budget:
                return False
        return True

    def _evict(self, nbytes, keep):
        idle = sorted((m for m in self.models.values() if not m.busy and m.id != keep), key=lambda m: m.last_used)
        freed = 0
        for m in idle:
            if freed >= nbytes:
                break
            freed += m.bytes
            self._destroy(m)
            del self.models[m.id]
            self.evicted.add(m.id)
            self.evictions += 1

    def _destroy(self, m):
        for attr in ("h", "hvg"):
            h = getattr(m, attr)
            if h:
                self.lib.pgb_gp_destroy(h)
                setattr(m, attr, None)
        self.used -= m.bytes
        m.bytes = 0

    def _take(self, role, scan=64):
        """Called with the lock held: the next runnable request, or None.

        "small" workers take only small requests, "small_first" workers look
        at the small requests first, "any" workers take the earliest arrival
        of either class.  Up to `scan` requests whose model is busy (or that
        do not fit in memory yet) are stepped over and put back."""
        skipped = []
        found = None
        large_ok = not self.max_large or self.large_running < self.max_large
        for _ in range(scan):
            heaps = self.heaps
            big = heaps[1] if large_ok else []
            if role == "small":
                h = heaps[0]
            elif role == "small_first":
                h = heaps[0] if heaps[0] else big
            elif heaps[0] and big:
                h = heaps[0] if heaps[0][0] < big[0] else big
            else:
                h = heaps[0] if heaps[0] else big
            if not h:
                break
            item = heapq.heappop(h)
            req = item[2]
            if req.kind == "predict" and req.model in self.evicted and req.model not in self.models:
                req.error = "model evicted before the request"
                req.start = req.done = self.now()
                self.lock.notify_all()
                continue
            if self._runnable(req):
                found = req
                break
            skipped.append((h, item))
        for h, item in skipped:
            heapq.heappush(h, item)
        if found is None:
            return None
        req = found
        m = self.models.get(req.model)
        if m is None:
            m = _Model(req.model, req.problem)
            self.models[req.model] = m
        m.busy = True
        if req.n > self.small_n:
            self.large_running += 1
        fit, vg, cap = self._plan(req, m)
        grow = m.footprint(fit, vg, cap) - m.bytes
        self.used += grow
        m.bytes += grow
        return req, m

    # -- execution ----------------------------------------------------------------
    def _worker(self, streams, role):
        torch = self.torch
        torch.cuda.set_device(self.device)
        while True:
            with self.lock:
                while True:
                    if self.stop and not self._pending():
                        return
                    got = self._take(role)
                    if got is not None:
                        self.busy_workers += 1   # counted before the lock is released (wait_idle)
                        break
                    self.lock.wait(timeout=0.002)
            req, m = got
            stream = streams[0] if req.n <= self.small_n else streams[1]
            req.start = self.now()
            try:
                with torch.cuda.stream(stream):
                    self._run(req, m, stream)
                stream.synchronize()
            except Exception as exc:   # reported per request
                req.error = repr(exc)
            req.done = self.now()
            if req.n > self.small_n:
                with self.lock:
                    self.large_running -= 1
                    self.lock.notify_all()
            warm = (req.kind == "fit" and req.error is None and m.hvg is None
                    and (self.warm_large if m.problem.n > self.small_n else self.warm_small))
            with self.lock:
                if warm:   # account the handles first; skip the warm-up if they do not fit
                    cap = max(m.cap_m, -(-self.warm_rows // 128) * 128)
                    grow = m.footprint(True, True, cap) - m.bytes
                    warm = self.used + grow <= self.budget
                    if warm:
                        self.used += grow
                        m.bytes += grow
                        m.cap_m = cap
                if not warm:
                    m.busy = False
                    m.last_used = req.done
                if req.kind == "predict" and req.error is None:
                    m.cap_m = max(m.cap_m, -(-req.Xs.shape[0] // 128) * 128)
                self.lock.notify_all()
            if warm:
                try:
                    with torch.cuda.stream(stream):
                        self._warm_vg(m, stream)
                    stream.synchronize()
                except Exception as exc:   # the first request on the model creates it instead
                    self.warm_errors.append((m.id, repr(exc)))
                with self.lock:
                    m.busy = False
                    m.last_used = self.now()
                    self.lock.notify_all()
            with self.lock:
                self.busy_workers -= 1
                self.lock.notify_all()

    def _upload(self, m):
        torch = self.torch
        p = m.problem
        if "X" not in m.dev:
            ydt = torch.int32 if p.J else torch.float32
            m.dev["X"] = torch.from_numpy(np.ascontiguousarray(p.X, np.float32)).to(self.device, non_blocking=True)
            m.dev["y"] = torch.from_numpy(np.ascontiguousarray(p.y)).to(self.device, ydt, non_blocking=True)

    def _create(self, p):
        h = C.c_void_p()
        N.check(self.lib.pgb_gp_create(p.desc(), C.byref(h)), "pgb_gp_create")
        cap = self.large_blocks if p.n > self.small_n else self.small_blocks
        if cap:
            N.check(self.lib.pgb_gp_set_max_blocks(h, cap), "pgb_gp_set_max_blocks")
        return h

    def _warm_vg(self, m, stream):
        """Create the model's evidence + gradient handle and capture its graph
        (one evaluation at the fitted hyperparameters), and size the fit
        handle's predict workspace for m.cap_m rows (one prediction at the
        training inputs' first row, repeated); the results are dropped."""
        torch = self.torch
        p = m.problem
        if m.hvg is None:
            m.hvg = self._create(p)
        d = m.dev
        theta = torch.from_numpy(np.asarray(p.theta, np.float32)).to(self.device, non_blocking=True)
        out = torch.empty(1 + theta.numel(), dtype=torch.float32, device=self.device)
        N.check(self.lib.pgb_value_and_grad(m.hvg, d["X"].data_ptr(), d["y"].data_ptr(), theta.data_ptr(),
                                            out.data_ptr(), out[1:].data_ptr(), stream.cuda_stream), "warm-up")
        M = m.cap_m
        if M > 0:
            Xs = d["X"][:1].expand(M, -1).contiguous()
            mean = torch.empty(M, dtype=torch.float32, device=self.device)
            var = torch.empty_like(mean)
            N.check(self.lib.pgb_predict(m.h, d["X"].data_ptr(), d["theta"].data_ptr(), d["a"].data_ptr(),
                                         d["W"].data_ptr(), Xs.data_ptr(), M, mean.data_ptr(), var.data_ptr(), 1,
                                         stream.cuda_stream), "warm-up predict")

    def _run(self, req, m, stream):
        torch = self.torch
        lib = self.lib
        sh = stream.cuda_stream
        p = req.problem
        dev = self.device
        self._upload(m)
        d = m.dev
        if req.kind == "fit":
            if m.h is None:
                m.h = self._create(p)
                d["a"] = torch.empty(p.n, dtype=torch.float32, device=dev)
                d["W"] = torch.empty(p.n, dtype=torch.float32, device=dev)
            d["theta"] = torch.from_numpy(np.asarray(p.theta, np.float32)).to(dev, non_blocking=True)
            N.check(lib.pgb_approximate_posterior(m.h, d["X"].data_ptr(), d["y"].data_ptr(), d["theta"].data_ptr(),
                                                  d["a"].data_ptr(), d["W"].data_ptr(), sh), "fit")
            a = d["a"].to("cpu", non_blocking=True)
            stream.synchronize()
            m.fitted = True
            req.result = (a.numpy(),)
        elif req.kind == "vg":
            if m.hvg is None:
                m.hvg = self._create(p)
            th = req.theta if req.theta is not None else p.theta
            theta = torch.from_numpy(np.asarray(th, np.float32)).to(dev, non_blocking=True)
            out = torch.empty(1 + theta.numel(), dtype=torch.float32, device=dev)
            N.check(lib.pgb_value_and_grad(m.hvg, d["X"].data_ptr(), d["y"].data_ptr(), theta.data_ptr(),
                                           out.data_ptr(), out[1:].data_ptr(), sh), "value_and_grad")
            host = out.to("cpu", non_blocking=True)
            stream.synchronize()
            req.result = (float(host[0]), host[1:].numpy())
        else:
            Xs = torch.from_numpy(np.ascontiguousarray(req.Xs, np.float32)).to(dev, non_blocking=True)
            M = Xs.shape[0]
            mean = torch.empty(M, dtype=torch.float32, device=dev)
            var = torch.empty(M, dtype=torch.float32, device=dev)
            N.check(lib.pgb_predict(m.h, d["X"].data_ptr(), d["theta"].data_ptr(), d["a"].data_ptr(),
                                    d["W"].data_ptr(), Xs.data_ptr(), M, mean.data_ptr(), var.data_ptr(), 1, sh),
                    "predict")
            mh, vh = mean.to("cpu", non_blocking=True), var.to("cpu", non_blocking=True)
            stream.synchronize()
            req.result = (mh.numpy(), vh.numpy())

    def wait_idle(self):
        """Block until no request is queued and every worker is idle (warm-ups
        included)."""
        with self.lock:
            while self._pending() or self.busy_workers:
                self.lock.wait(timeout=0.01)

    # -- open-loop replay --------------------------------------------------------
    def replay(self, requests, realtime=True):
        """Submit `requests` at their arrival times (seconds from now) and wait
        for all of them; returns the requests with start/done times filled."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        self.t0 = time.perf_counter()
        for r in reqs:
            if realtime:
                delay = r.arrival - self.now()
                if delay > 0:
                    time.sleep(delay)
            self.submit(r)
        while True:
            with self.lock:
                if all(r.done is not None for r in reqs):
                    break
                self.lock.wait(timeout=0.01)
        return reqs


def latency_summary(reqs, small_n=2048):
    """p50 / p99 latency (ms) of all requests, per kind, and of n <= small_n."""
    def pct(xs):
        if not xs:
            return None
        xs = np.sort(np.asarray(xs)) * 1e3
        return {"p50_ms": float(np.percentile(xs, 50)), "p99_ms": float(np.percentile(xs, 99)),
                "mean_ms": float(xs.mean()), "count": int(xs.size)}

    ok = [r for r in reqs if r.error is None and r.done is not None]
    out = {"all": pct([r.latency for r in ok]),
           "service_all": pct([r.done - r.start for r in ok]),
           f"n<={small_n}": pct([r.latency for r in ok if r.n <= small_n])}
    for k in ("fit", "vg", "predict"):
        out[k] = pct([r.latency for r in ok if r.kind == k])
    span = max(r.done for r in ok) - min(r.arrival for r in reqs) if ok else 0.0
    out["throughput_req_s"] = len(ok) / span if span > 0 else None
    out["errors"] = sum(1 for r in reqs if r.error is not None)
    return out
