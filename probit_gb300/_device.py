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


def as_device(x, dtype, device=None):
    """Contiguous CUDA tensor of `dtype` holding `x` (copied only if needed)."""
    torch = _torch()
    dev = device if device is not None else require_cuda()
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
