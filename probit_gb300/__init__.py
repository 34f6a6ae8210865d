"""probit_gb300: GB300-native (sm_103a) approximate inference for GPs.

A drop-in for the approximate-inference path of the reference package
(bb515/probit): ``LaplaceGP`` and ``VBGP`` with ``weight``, ``precision``,
``approximate_posterior``, ``objective``, ``value_and_grad``, ``predict`` and
``predict_covariance``; ``LaplaceBatch`` / ``ShardedBatch`` for many GPs of
any shapes, ``optimize.minimize_lockstep`` for their hyperparameter fits,
``serving.Server`` for request serving, ``autograd.evidence`` for torch
training loops and ``autotune`` for the factorisation's launch tuning —
computed by hand-written CUDA kernels behind the C-ABI declared in
``include/probit_gb300.h`` (raw device pointers) and
``include/probit_gb300_dlpack.h`` (DLPack tensors).
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
    "LaplaceGP", "VBGP", "LaplaceBatch", "ShardedBatch", "lpt_partition", "EQ", "Matern12",
    "log_gaussian_likelihood", "log_probit_likelihood", "log_probit_likelihood_stable",
    "grad_log_probit_likelihood", "hessian_log_probit_likelihood", "check_cutpoints", "check_data",
    "InvalidKernel", "probit_predictive_distributions",
]
__version__ = "0.1.0"
