"""CPU oracle for the Laplace approximate-inference path (TEST INFRASTRUCTURE).

This package restates, in NumPy/SciPy, the algorithm that the reference package
(bb515/probit) runs for ``LaplaceGP``: the dense-Jacobian Newton fixed point,
the negative log evidence, its implicit hyperparameter gradient and the
predictive mean/variance.  It is a checker, never the thing measured or
shipped: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` import it.  The product package ``probit_gb300`` never does.

Parity status: **unpinned**.  The reference is pure Python on JAX and needs
``jax``, ``jaxopt``, ``mlkernels`` and ``lab`` (``backends``), none of which is
installed or installable offline, so the reference cannot be run to produce
fixtures.  Its own test suite (``probit/test/test_implicit.py:11-22``) holds a
single known-answer test, for the tail-series polynomial ``h(x)``; that test is
reproduced against :func:`oracle.laplace.h` in ``tests/test_oracle.py``.  The
rest of the oracle is pinned by analytic identities instead (closed-form GP
marginal likelihood for the Gaussian likelihood, the Woodbury equivalence of
the reference's LU Newton step and the B = I + W^1/2 K W^1/2 form, central
finite differences of the full objective for the gradient).

Third-party arithmetic restated here (not vendored in the reference):

* mlkernels >= 0.3.6 (``setup.py:41``): ``EQ`` = exp(-r^2/2), ``Matern12`` =
  exp(-r), ``k.stretch(l)`` divides the inputs by ``l``, ``k.periodic(p)`` maps
  each input coordinate x to (sin 2*pi*x/p, cos 2*pi*x/p), ``s * k`` scales.
* lab / backends >= 1.4.32 (``setup.py:40``): pairwise distances, cholesky,
  solve.  The exact form of lab's pairwise distance is not available offline;
  the default here is the difference form, and ``distance="expanded"``
  restates the |a|^2 + |b|^2 - 2 a.b form (clamped at 0, sqrt floor 1e-12)
  as a compatibility mode.
* jaxopt >= 0.5.5 (``setup.py:39``): ``FixedPointIteration`` with maxiter 100,
  stopping when ||z_k - z_{k-1}||_2 <= tol, at most maxiter updates.
"""

from .laplace import *  # noqa: F401,F403
