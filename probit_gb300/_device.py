"""Device plumbing: torch tensors are used only for device memory and streams."""

from __future__ import annotations

import numpy as np


def _torch():
    import torch

    return torch


def require_cuda():
    """The CUDA device the library runs on; raises when there is none."""
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("probit_gb300 needs a CUDA device (sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def from_dlpack_or_none(x):
    """A torch view of an array from another framework that speaks DLPack
    (a JAX or CuPy array: no copy when it is already on the device), or None
    for torch tensors, NumPy arrays, Python objects and producers torch
    cannot import."""
    torch = _torch()
    if isinstance(x, (torch.Tensor, np.ndarray)) or not hasattr(x, "__dlpack__"):
        return None
    try:
        return torch.from_dlpack(x)
    except (TypeError, ValueError, RuntimeError, BufferError):
        return None


def as_device(x, dtype, device=None):
    """Contiguous CUDA tensor of `dtype` holding `x` (copied only if needed;
    DLPack arrays of other frameworks are taken without a host round trip)."""
    torch = _torch()
    dev = device if device is not None else require_cuda()
    t = from_dlpack_or_none(x)
    if t is not None:
        x = t
    if isinstance(x, torch.Tensor):
        t = x.detach()
        if t.device != dev or t.dtype != dtype:
            t = t.to(device=dev, dtype=dtype, non_blocking=True)
        return t.contiguous()
    arr = np.ascontiguousarray(np.asarray(x))
    t = torch.from_numpy(arr)
    return t.to(device=dev, dtype=dtype).contiguous()


def stream_handle(device=None) -> int:
    """cudaStream_t of torch's current stream on `device`, as an integer."""
    torch = _torch()
    return torch.cuda.current_stream(device).cuda_stream


def like_input(t, ref):
    """Return `t` as a torch tensor when `ref` is one, else as a NumPy array."""
    torch = _torch()
    if isinstance(ref, torch.Tensor):
        return t
    return t.cpu().numpy()
