"""Small helpers shared by the host-side modules: device pointers, streams, checks."""
from __future__ import annotations

import ctypes

import torch


def require_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("tensorf_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU fallback")


def stream_handle(stream: torch.cuda.Stream | None = None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def ptr(t: torch.Tensor | None, dtype: torch.dtype | None = None, name: str = "tensor") -> ctypes.c_void_p:
    """Device pointer of a contiguous CUDA tensor (NULL for None)."""
    if t is None:
        return ctypes.c_void_p(0)
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    return ctypes.c_void_p(t.data_ptr())


def workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
