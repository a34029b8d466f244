"""Device buffers and streams for the C-ABI calls (PyTorch used only as an allocator)."""
from __future__ import annotations

import numpy as np
import torch


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("pygw_gb300: the GB300 path needs a CUDA device; there is no CPU fallback")


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def stream_handle(stream=None) -> int:
    s = torch.cuda.current_stream() if stream is None else stream
    return s.cuda_stream


def to_device(a, dtype=None):
    """numpy array or tensor → contiguous CUDA tensor (C order of the given array)."""
    if isinstance(a, torch.Tensor):
        t = a if a.is_cuda else a.cuda(non_blocking=True)
        if dtype is not None and t.dtype != dtype:
            t = t.to(dtype)
        return t.contiguous()
    arr = np.ascontiguousarray(a)
    t = torch.from_numpy(arr)
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def workspace(nbytes: int):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")


def free_device_bytes() -> int:
    """Device memory a new allocation can use: what the driver reports free
    plus what PyTorch's caching allocator holds reserved but unused (after a
    large call the allocator keeps its blocks, which the driver counts as in
    use; sizing the next call on the driver's figure alone would shrink it)."""
    free, _ = torch.cuda.mem_get_info()
    return int(free + torch.cuda.memory_reserved() - torch.cuda.memory_allocated())
