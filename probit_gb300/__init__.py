"""probit_gb300: GB300-native (sm_103a) Laplace approximate inference for GPs.

A drop-in for the Laplace path of the reference package (bb515/probit):
``LaplaceGP`` with ``weight``, ``precision``, ``approximate_posterior``,
``objective``, ``value_and_grad`` and ``predict``, computed by hand-written
CUDA kernels behind the C-ABI declared in ``include/probit_gb300.h``.
"""

from .approximators import LaplaceGP, VBGP
from .batch import LaplaceBatch
from .shard import ShardedBatch, lpt_partition
from .kernels import EQ, Matern12
from .utilities import (
    InvalidKernel,
    check_cutpoints,
    check_data,
    grad_log_probit_likelihood,
    hessian_log_probit_likelihood,
    log_gaussian_likelihood,
    log_probit_likelihood,
    log_probit_likelihood_stable,
    probit_predictive_distributions,
)

__all__ = [
    "LaplaceGP", "VBGP", "LaplaceBatch", "ShardedBatch", "lpt_partition", "EQ", "Matern12", "log_gaussian_likelihood", "log_probit_likelihood",
    "log_probit_likelihood_stable", "grad_log_probit_likelihood", "hessian_log_probit_likelihood",
    "check_cutpoints", "check_data", "InvalidKernel", "probit_predictive_distributions",
]
__version__ = "0.1.0"
