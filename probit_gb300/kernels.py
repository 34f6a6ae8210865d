"""Kernel specifications with mlkernels' composition syntax.

The reference builds its prior with mlkernels (``prior(params) -> kernel``;
``approximators.py:69-71``, ``examples/regression.py:120-123``,
``examples/classification.py:389-391``).  mlkernels is not a dependency
here; these small objects accept the same expressions for the families the
CUDA kernels implement:

    s * EQ().stretch(l)                 s * Matern12().stretch(l)
    s * EQ().stretch(l).periodic(p)

``l`` is a scalar or a length-D vector (ARD); ``s`` and ``l`` may be Python
numbers, NumPy arrays or torch tensors (torch tensors keep their autograd
graph, which is how gradients reach arbitrary ``params`` pytrees).  Anything
outside these families raises ``NotImplementedError``.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

KIND_EQ = "eq"
KIND_MATERN12 = "matern12"
KIND_EQ_PERIODIC = "eq_periodic"


@dataclass(frozen=True)
class KernelSpec:
    """A resolved kernel: family, lengthscale(s), signal variance, period."""

    kind: str
    lengthscale: Any = 1.0
    variance: Any = 1.0
    period: float | None = None


@dataclass
class Kernel:
    """A stationary kernel under construction (EQ or Matern12 base)."""

    base: str
    scale: Any = 1.0
    ell: Any = None
    period: float | None = None
    _ops: tuple = field(default_factory=tuple)

    # -- composition ----------------------------------------------------
    def stretch(self, lengthscale) -> "Kernel":
        if self.ell is not None:
            raise NotImplementedError("a kernel can be stretched once")
        if self.period is not None:
            raise NotImplementedError(
                "k.periodic(p).stretch(l) is not supported; use k.stretch(l).periodic(p)")
        return Kernel(self.base, self.scale, lengthscale, None, self._ops + ("stretch",))

    def periodic(self, period) -> "Kernel":
        if self.base != KIND_EQ:
            raise NotImplementedError("periodic() is supported on EQ only")
        if self.period is not None:
            raise NotImplementedError("a kernel can be made periodic once")
        return Kernel(self.base, self.scale, self.ell, float(period), self._ops + ("periodic",))

    def __mul__(self, other) -> "Kernel":
        if isinstance(other, Kernel):
            raise NotImplementedError("products of kernels are not supported")
        return Kernel(self.base, _mul(self.scale, other), self.ell, self.period, self._ops)

    __rmul__ = __mul__

    def __add__(self, other):
        raise NotImplementedError("sums of kernels are not supported")

    __radd__ = __add__

    def spec(self) -> KernelSpec:
        kind = self.base
        if self.period is not None:
            kind = KIND_EQ_PERIODIC
        ell = 1.0 if self.ell is None else self.ell
        return KernelSpec(kind, ell, self.scale, self.period)


def _mul(a, b):
    if isinstance(a, (int, float)) and a == 1.0:
        return b
    if isinstance(b, (int, float)) and b == 1.0:
        return a
    return a * b


def EQ() -> Kernel:
    """Exponentiated quadratic, k(r) = exp(-r^2 / 2)."""
    return Kernel(KIND_EQ)


def Matern12() -> Kernel:
    """Matern-1/2 (exponential), k(r) = exp(-r)."""
    return Kernel(KIND_MATERN12)


def resolve(kernel) -> KernelSpec:
    """KernelSpec of a kernel object returned by a user's ``prior`` callable."""
    if isinstance(kernel, KernelSpec):
        return kernel
    if isinstance(kernel, Kernel):
        return kernel.spec()
    raise NotImplementedError(
        f"{type(kernel).__name__} is not a supported kernel; build the prior from "
        "probit_gb300.kernels.EQ / Matern12 with stretch, periodic and scaling")
