"""Device memory and streams for the evaluators (PyTorch is used as the CUDA allocator only).

Tables and hash tables live in torch CUDA tensors whose data pointers are handed to the C-ABI;
the library runs its kernels on the current torch stream.  Without a GPU every evaluator raises:
there is no CPU path in this package.
"""
from __future__ import annotations

import torch


class NoGPUError(RuntimeError):
    pass


def require_gpu():
    if not torch.cuda.is_available():
        raise NoGPUError("tropidist_gb300 evaluators run on the GPU only; no CUDA device is visible")


def empty(nbytes, dtype=torch.uint8):
    require_gpu()
    n = max(1, int(nbytes) // torch.empty(0, dtype=dtype).element_size())
    return torch.empty(n, dtype=dtype, device="cuda")


def ptr(t):
    return t.data_ptr() if t is not None else None


def stream_ptr():
    return torch.cuda.current_stream().cuda_stream


def free_bytes():
    require_gpu()
    free, _total = torch.cuda.mem_get_info()
    return free
