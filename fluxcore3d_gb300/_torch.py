"""Tensor plumbing between torch (device memory, streams) and the C ABI."""
from __future__ import annotations

import torch


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def require(t: torch.Tensor, name: str, dtype: torch.dtype | None = None, numel: int | None = None) -> None:
    """Validation matching the reference's TORCH_CHECK messages (CUDA, contiguous, dtype)."""
    if not isinstance(t, torch.Tensor):
        raise RuntimeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be on CUDA")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise RuntimeError(f"{name} must be {str(dtype).replace('torch.', '')}")
    if numel is not None and t.numel() != numel:
        raise RuntimeError(f"{name} must have {numel} elements")


def capture_graph(fn):
    """CUDA graph of fn() with Python's cyclic garbage collector paused during the capture.

    Solver objects that own captured graphs sit in reference cycles, so only the cyclic
    collector frees them; a collection triggered inside another capture would destroy their
    graphs there, and a graph may not be reset while a stream captures (the capture is then
    invalidated).  torch.cuda.graph collects once on entry, before the capture begins."""
    import gc
    g = torch.cuda.CUDAGraph()
    was = gc.isenabled()
    gc.disable()
    try:
        with torch.cuda.graph(g):
            fn()
    finally:
        if was:
            gc.enable()
    return g
