"""Device plumbing: torch tensors as the owners of device memory and streams."""
from __future__ import annotations

import numpy as np
import torch


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("gala_gb300 needs a CUDA device: no GPU is visible to torch")
    return torch.device("cuda", torch.cuda.current_device())


def stream_handle(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def as_device_f64(a, device=None) -> torch.Tensor:
    """Contiguous float64 CUDA tensor view/copy of ``a`` (numpy, list or tensor)."""
    dev = device or require_cuda()
    if isinstance(a, torch.Tensor):
        # a pinned host tensor is copied asynchronously on the current stream
        nb = a.device.type == "cpu" and a.is_pinned()
        return a.to(device=dev, dtype=torch.float64, non_blocking=nb).contiguous()
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if not arr.flags.writeable:
        arr = arr.copy()
    return torch.from_numpy(arr).to(dev)


def ptr(t: torch.Tensor) -> int:
    return int(t.data_ptr())
