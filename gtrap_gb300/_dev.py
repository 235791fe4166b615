"""Device-memory plumbing shared by the drop-in modules.

PyTorch provides device memory, streams and copies; the computation itself is in
the native library.  Pointers may be given as ``driver.DeviceAllocation`` objects,
CUDA torch tensors or plain integers (raw device addresses).
"""
from __future__ import annotations

import threading

import numpy as np
import torch

_ws_lock = threading.Lock()
_workspaces: dict = {}


def require_cuda():
    if not torch.cuda.is_available():
        from ._native import GtrapError, ERR_UNSUPPORTED
        raise GtrapError(ERR_UNSUPPORTED, "gtrap_gb300 needs a CUDA device; none is visible")


def as_ptr(obj) -> int:
    """Raw device address of a pointer-like argument (None -> 0)."""
    if obj is None:
        return 0
    if isinstance(obj, torch.Tensor):
        if not obj.is_cuda:
            raise TypeError("expected a CUDA tensor, got a tensor on %s" % obj.device)
        if not obj.is_contiguous():
            raise ValueError("device tensors passed to gtrap_gb300 must be contiguous")
        return obj.data_ptr()
    if isinstance(obj, (int, np.integer)):
        return int(obj)
    ptr = getattr(obj, "ptr", None)
    if ptr is not None:
        return int(ptr)
    return int(obj)


def stream_handle(stream=None) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    handle = getattr(stream, "handle", None)
    if handle is not None:
        return int(handle)
    return int(stream)


def workspace(nbytes: int, device=None, slot: str = "default", stream=None) -> torch.Tensor:
    """A cached device scratch buffer of at least ``nbytes`` (256-byte aligned) for launches on
    ``stream`` (default: the current stream).

    Buffers are cached per (device, slot, launch stream), so calls on one stream reuse a buffer
    in stream order and calls on different streams never share one.  The buffer is allocated
    on the current stream: a caller that launches on another stream keeps that stream's work
    ordered after the current stream's (or makes it current, ``with torch.cuda.stream(s)``),
    as it must for the output tensors the API functions allocate there too.
    """
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    launch = stream_handle(stream) if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    key = (dev.index, slot, launch)
    with _ws_lock:
        buf = _workspaces.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
            _workspaces[key] = buf
    return buf


def release_workspaces():
    with _ws_lock:
        _workspaces.clear()
