"""A small ``pycuda.driver`` stand-in so reference-style driver code runs unchanged.

The reference allocates with ``cuda.mem_alloc`` and moves data with the synchronous
``cuda.memcpy_htod`` / ``cuda.memcpy_dtoh`` (e.g. ``ipynb/example geebls  Kepler
Planet.ipynb`` cell 13, ``kepler/gtls_mockkepler.py:280-318``).  Here the memory is a
PyTorch CUDA buffer and copies run on the current PyTorch stream and complete before
returning, as in PyCUDA.
"""
from __future__ import annotations

import numpy as np
import torch

from ._dev import as_ptr, require_cuda


class DeviceAllocation:
    """Device buffer of ``nbytes`` bytes; ``int(alloc)`` is its device address."""

    def __init__(self, nbytes: int):
        require_cuda()
        self.nbytes = int(nbytes)
        self._buf = torch.empty(max(self.nbytes, 1), dtype=torch.uint8, device="cuda")

    @property
    def ptr(self) -> int:
        return self._buf.data_ptr()

    def __int__(self) -> int:
        return self.ptr

    def __index__(self) -> int:
        return self.ptr

    def as_tensor(self, dtype=torch.uint8, count=None) -> torch.Tensor:
        """View of the buffer as a flat tensor of ``dtype``."""
        item = torch.empty((), dtype=dtype).element_size()
        n = self.nbytes // item if count is None else int(count)
        return self._buf[: n * item].view(dtype)

    def free(self):
        self._buf = torch.empty(1, dtype=torch.uint8, device=self._buf.device)
        self.nbytes = 0


def mem_alloc(nbytes) -> DeviceAllocation:
    return DeviceAllocation(int(nbytes))


def _bytes_of(array: np.ndarray) -> torch.Tensor:
    a = np.ascontiguousarray(array)
    return torch.from_numpy(a.reshape(-1).view(np.uint8))


def _dev_bytes(dest, nbytes) -> torch.Tensor:
    if isinstance(dest, DeviceAllocation):
        if nbytes > dest.nbytes:
            raise ValueError("copy of %d bytes exceeds allocation of %d" % (nbytes, dest.nbytes))
        return dest._buf[:nbytes]
    if isinstance(dest, torch.Tensor):
        return dest.reshape(-1).view(torch.uint8)[:nbytes]
    raise TypeError("device side must be a DeviceAllocation or CUDA tensor (got %r)" % type(dest))


def memcpy_htod(dest, src):
    """Copy host array ``src`` to device buffer ``dest`` (blocking)."""
    host = _bytes_of(np.asarray(src))
    _dev_bytes(dest, host.numel()).copy_(host)
    torch.cuda.current_stream().synchronize()


def memcpy_dtoh(dest: np.ndarray, src):
    """Copy ``dest.nbytes`` bytes from device buffer ``src`` into host array ``dest``."""
    if not isinstance(dest, np.ndarray) or not dest.flags.c_contiguous:
        raise TypeError("memcpy_dtoh needs a C-contiguous numpy destination")
    view = torch.from_numpy(dest.reshape(-1).view(np.uint8))
    view.copy_(_dev_bytes(src, dest.nbytes))


def memset_d8(dest, value: int, count: int):
    _dev_bytes(dest, count).fill_(int(value) & 0xFF)


class Context:
    @staticmethod
    def synchronize():
        torch.cuda.synchronize()


def pointer(obj) -> int:
    """Device address of an allocation, tensor or integer."""
    return as_ptr(obj)
