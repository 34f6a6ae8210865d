"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py

For every case in cases.py the oracle (oracle/laplace.py, the NumPy
restatement of the reference algorithm) is run in float64 and in float32 on
the seeded inputs; inputs and outputs are saved to <case>.npz.  The
reference itself cannot run here (JAX is not installable offline), so these
fixtures pin the CUDA path to the oracle, and the oracle to the analytic
checks of tests/test_oracle.py.
"""

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE))

from cases import CASES, make, oracle_problem  # noqa: E402
from oracle import laplace as L  # noqa: E402


def run(name):
    p, theta, tol = make(name)
    lik = CASES[name][1]
    op = oracle_problem(p, lik)
    out = {"X": p.X, "y": p.y, "theta": theta, "tol": np.float64(tol), "Xtest": p.Xtest}
    for tag, dt in (("f64", np.float64), ("f32", np.float32)):
        op.X = p.X.astype(dt)
        v, g, a, it = L.value_and_grad(op, theta.astype(dt) if dt is np.float32 else theta, tol=tol, dtype=dt)
        W, f = L.precision(op, theta, a, dtype=dt)
        mean, var = L.predict(op, theta, p.Xtest.astype(dt), a, W, dtype=dt)
        out.update({f"value_{tag}": v, f"grad_{tag}": g, f"a_{tag}": a, f"iters_{tag}": np.int32(it),
                    f"W_{tag}": W, f"f_{tag}": f, f"mean_{tag}": mean, f"var_{tag}": var})
    np.savez_compressed(HERE / f"{name}.npz", **out)
    return out


if __name__ == "__main__":
    for name in CASES:
        o = run(name)
        print(f"{name:32s} iters f64={int(o['iters_f64'])} f32={int(o['iters_f32'])} "
              f"value={float(o['value_f64']):.6f} rel32={abs(o['value_f32']-o['value_f64'])/abs(o['value_f64']):.2e}")
