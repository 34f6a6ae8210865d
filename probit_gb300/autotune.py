"""Autotuner of the factorisation's launch shape per problem-size bucket.

The tile of the blocked Cholesky is fixed at 128 x 128 (the M = 128 shape
of the tcgen05 MMA that accumulates it) and its panel at 32 columns (one
warp); what changes the factorisation's speed with N is how much of each
column runs on the critical path.  The knob is the near band depth
(``pgb_gp_set_near_depth``): the tiles just below each diagonal tile that
are solved by substitution as the diagonal tile's panels appear, instead of
waiting for its inverse and using the tensor cores.  A deep band shortens
the critical path of long factorisations and costs substitution work; a
shallow one suits short factorisations, whose blocks are mostly idle.

``tune`` times candidate depths per bucket of tile counts (one Gaussian
evidence + gradient problem per bucket, seeded synthetic data) and returns a
``Table``; ``save`` / ``load`` keep it as JSON; ``use`` installs a table so
that ``LaplaceGP`` and ``LaplaceBatch`` set each new handle's depth from it.
The built-in rule (depth 3 from 16 tiles, else 2) applies where no table is
installed or a bucket has no entry.
"""

from __future__ import annotations

import json
import math
import os
import time
from dataclasses import dataclass, field
from pathlib import Path

# buckets of tile counts nt = ceil(N / 128): (lowest, highest)
BUCKETS = ((1, 2), (3, 4), (5, 8), (9, 16), (17, 32), (33, 64), (65, 1 << 20))
CANDIDATES = (1, 2, 3, 4, 6)
TILE = 128
ENV = "PGB_AUTOTUNE"


def builtin_depth(nt: int) -> int:
    """The library's built-in near band depth for an nt-tile factor."""
    return 3 if nt >= 16 else 2


def tiles(n: int) -> int:
    return -(-int(n) // TILE)


@dataclass
class Entry:
    lo: int              # tile counts lo .. hi
    hi: int
    depth: int           # chosen near band depth
    n: int               # problem size the bucket was timed at
    ms: dict             # depth -> median milliseconds per evaluation


@dataclass
class Table:
    device: str = ""
    entries: list = field(default_factory=list)

    def depth(self, n: int) -> int:
        """Near band depth for a problem of n points (0: the built-in rule)."""
        nt = tiles(n)
        for e in self.entries:
            if e.lo <= nt <= e.hi:
                return min(e.depth, max(1, nt - 1)) if nt > 1 else e.depth
        return 0

    def to_json(self) -> str:
        return json.dumps({"version": 1, "device": self.device,
                           "entries": [{"lo": e.lo, "hi": e.hi, "depth": e.depth, "n": e.n,
                                        "ms": {str(k): v for k, v in e.ms.items()}} for e in self.entries]},
                          indent=1)

    @classmethod
    def from_json(cls, text: str) -> "Table":
        d = json.loads(text)
        if d.get("version") != 1:
            raise ValueError("unknown autotune table version")
        ents = []
        for e in d["entries"]:
            depth = int(e["depth"])
            if not 1 <= depth <= 16 or int(e["lo"]) > int(e["hi"]):
                raise ValueError(f"bad autotune entry {e}")
            ents.append(Entry(int(e["lo"]), int(e["hi"]), depth, int(e["n"]),
                              {int(k): float(v) for k, v in e["ms"].items()}))
        return cls(str(d.get("device", "")), ents)


def bucket_size(lo: int, hi: int, cap_tiles: int = 64) -> int:
    """The problem size a bucket is timed at: the geometric middle of its
    tile counts (capped), in points."""
    hi = min(hi, max(lo, cap_tiles))
    return int(round(math.sqrt(lo * hi))) * TILE


def tune(time_fn, buckets=BUCKETS, candidates=CANDIDATES, max_tiles=64, device="") -> Table:
    """Pick the fastest near band depth per bucket.  ``time_fn(n, depth)``
    returns the time of one evaluation at n points with that depth (any
    unit; smaller is better).  Depths deeper than the factor has tiles
    below the diagonal are not tried; ties keep the shallower depth."""
    table = Table(device=device)
    for lo, hi in buckets:
        if lo > max_tiles:
            break
        n = bucket_size(lo, hi, max_tiles)
        nt = tiles(n)
        ms = {}
        for q in candidates:
            if q > max(1, nt - 1) and q != min(candidates):
                continue
            ms[q] = float(time_fn(n, q))
        best = min(sorted(ms), key=lambda q: ms[q])
        table.entries.append(Entry(lo, hi, best, n, ms))
    return table


def gpu_timer(reps: int = 5, warmup: int = 2, seed: int = 0):
    """``time_fn`` for ``tune``: median milliseconds of one Gaussian EQ
    evidence + gradient evaluation (D = 4, ARD) through the C-ABI, timed
    with CUDA events on the calling stream."""
    import ctypes as C

    import numpy as np
    import torch

    from . import _native as N
    from . import workloads as W

    lib = N.load()
    dev = torch.device("cuda", torch.cuda.current_device())

    def time_fn(n, depth):
        rng = np.random.default_rng(seed + n)
        p = W.regression_problem(rng, n, 4, "eq", np.array([0.5, 1.0, 1.5, 2.0]), 1.0, 0.2)
        desc = N.Desc(n, 4, N.KERNEL_EQ, 4, 1.0, N.LIK_GAUSSIAN, 0, 1e-5, 100, 0)
        h = C.c_void_p()
        N.check(lib.pgb_gp_create(desc, C.byref(h)), "pgb_gp_create")
        try:
            N.check(lib.pgb_gp_set_near_depth(h, int(depth)), "pgb_gp_set_near_depth")
            X = torch.tensor(np.asarray(p.X, np.float32), device=dev)
            y = torch.tensor(np.asarray(p.y, np.float32), device=dev)
            th = torch.tensor(p.theta().astype(np.float32), device=dev)
            v = torch.empty(1, device=dev)
            g = torch.empty(th.numel(), device=dev)
            s = torch.cuda.current_stream()
            call = lambda: N.check(lib.pgb_value_and_grad(h, X.data_ptr(), y.data_ptr(), th.data_ptr(),
                                                          v.data_ptr(), g.data_ptr(), s.cuda_stream),
                                   "pgb_value_and_grad")
            for _ in range(warmup):
                call()
            times = []
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                call()
                b.record(s)
                b.synchronize()
                times.append(a.elapsed_time(b))
            return float(np.median(times))
        finally:
            torch.cuda.synchronize()
            lib.pgb_gp_destroy(h)

    return time_fn


def default_path() -> Path:
    return Path(__file__).resolve().parent / "_lib" / "autotune.json"


def save(table: Table, path=None) -> Path:
    p = Path(path) if path else default_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(table.to_json())
    os.replace(tmp, p)
    return p


def load(path=None) -> Table | None:
    p = Path(path) if path else default_path()
    if not p.exists():
        return None
    return Table.from_json(p.read_text())


_installed: Table | None = None
_env_checked = False


def use(table: Table | None) -> None:
    """Install `table` for the handles created from now on (None: the
    built-in rule)."""
    global _installed, _env_checked
    _installed = table
    _env_checked = True


def current() -> Table | None:
    """The installed table; on first use, the one named by $PGB_AUTOTUNE
    (a JSON path) if set."""
    global _installed, _env_checked
    if not _env_checked:
        _env_checked = True
        path = os.environ.get(ENV)
        if path:
            _installed = load(path)
    return _installed


def depth_for(n: int) -> int:
    """Near band depth for a new handle of n points (0: built-in rule)."""
    t = current()
    return t.depth(n) if t is not None else 0


def main(argv=None) -> int:
    """``python -m probit_gb300.autotune [--out PATH] [--max-tiles T] [--reps R]``:
    tune on the current GPU and save the table."""
    import argparse

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--out", default=None)
    ap.add_argument("--max-tiles", type=int, default=64)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    import torch

    t0 = time.time()
    table = tune(gpu_timer(reps=a.reps), max_tiles=a.max_tiles, device=torch.cuda.get_device_name())
    path = save(table, a.out)
    for e in table.entries:
        print(f"tiles {e.lo}..{e.hi} (n={e.n}): depth {e.depth}  " +
              "  ".join(f"{q}:{ms:.3f}" for q, ms in sorted(e.ms.items())))
    print(f"saved {path} in {time.time() - t0:.1f} s")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
