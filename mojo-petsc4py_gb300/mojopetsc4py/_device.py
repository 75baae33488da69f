"""Device memory, copies and streams for the PETSc classes.

Everything goes through libgpetsc.so's own entry points (gp_device_alloc,
gp_host_alloc, gp_copy, gp_stream_synchronize), so `from mojopetsc4py import
PETSc` needs no other CUDA binding; PyTorch is imported only by the autograd
wrapper (adjoint.py), through `torch()` below.

Streams: each call is queued on the caller's current stream -- torch's
current CUDA stream when the process has imported torch (so the work orders
with the caller's torch code), else the default stream.  The two agree until
the caller selects another torch stream.

Device blocks expose __cuda_array_interface__ (version 3): torch, CuPy or
Numba view them without a copy (`torch.as_tensor(block, device="cuda")`).
"""

from __future__ import annotations

import ctypes
import sys

import numpy as np

from ._lib import check, device_count, lib

_has_device = None


def has_device() -> bool:
    global _has_device
    if _has_device is None:
        _has_device = device_count() > 0
    return _has_device


def require_device() -> None:
    if not has_device():
        raise RuntimeError("mojopetsc4py (GB300 build) needs a CUDA device; none is visible")


def torch():
    """PyTorch with a CUDA device (the autograd wrapper's dependency)."""
    import torch as t

    if not t.cuda.is_available():
        raise RuntimeError("mojopetsc4py (GB300 build) needs a CUDA device; torch sees none")
    return t


def stream_ptr() -> int:
    """The caller's current CUDA stream, as the void* the C ABI takes (0 is the
    default stream)."""
    t = sys.modules.get("torch")
    cuda = getattr(t, "cuda", None) if t is not None else None
    if cuda is not None and cuda.is_initialized():
        return int(cuda.current_stream().cuda_stream)
    return 0


def synchronize() -> None:
    """Wait for the work queued on the current stream."""
    check(lib().gp_stream_synchronize(stream_ptr()))


class DeviceArray:
    """A C-contiguous array in device memory from the library's stream-ordered
    pool.  The block is freed, ordered on the stream it was allocated on, when
    the object goes away."""

    __slots__ = ("ptr", "shape", "dtype", "_stream", "__weakref__")

    def __init__(self, shape, dtype=np.float64):
        self.ptr = 0
        self.shape = (int(shape),) if np.ndim(shape) == 0 else tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        if any(s < 0 for s in self.shape):
            raise ValueError("negative dimension")
        require_device()
        self._stream = stream_ptr()
        p = ctypes.c_void_p()
        check(lib().gp_device_alloc(ctypes.byref(p), self.nbytes, self._stream))
        self.ptr = p.value or 0

    @property
    def size(self) -> int:
        return int(np.prod(self.shape, dtype=np.int64))

    @property
    def nbytes(self) -> int:
        return self.size * self.dtype.itemsize

    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": self.dtype.str, "data": (self.ptr, False),
                "strides": None, "version": 3}

    def copy_from_host(self, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a, dtype=self.dtype)
        if a.size != self.size:
            raise ValueError(f"size mismatch: {a.size} into {self.size}")
        upload(self.ptr, a)
        return self

    def to_host(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape, dtype=self.dtype)
        download(out, self.ptr)
        return out

    def __del__(self):
        if self.ptr:
            try:
                lib().gp_device_free(self.ptr, self._stream)
            except Exception:
                pass
            self.ptr = 0


def empty(n, dtype=np.float64) -> DeviceArray:
    return DeviceArray(n, dtype)


def from_host(a: np.ndarray) -> DeviceArray:
    a = np.ascontiguousarray(a)
    return DeviceArray(a.shape, a.dtype).copy_from_host(a)


def upload(dst: int, a: np.ndarray) -> None:
    """Copy the C-contiguous host array `a` to device address `dst` and wait."""
    if a.nbytes:
        check(lib().gp_copy(dst, a.ctypes.data, a.nbytes, 1, stream_ptr()))


def download(a: np.ndarray, src: int) -> None:
    """Wait for the queued work, then copy device address `src` into the
    C-contiguous host array `a`."""
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("download needs a C-contiguous host array")
    if a.nbytes:
        check(lib().gp_copy(a.ctypes.data, src, a.nbytes, 1, stream_ptr()))


def device_view(a):
    """(pointer, shape, dtype) of a C-contiguous device array -- a DeviceArray
    or anything with __cuda_array_interface__, such as a CUDA torch tensor --
    or None when `a` is not a device array.  Raises ValueError for a strided
    device array."""
    if isinstance(a, DeviceArray):
        return a.ptr, a.shape, a.dtype
    try:
        cai = a.__cuda_array_interface__
    except (AttributeError, TypeError):
        return None
    except RuntimeError:  # a torch tensor that requires grad
        cai = a.detach().__cuda_array_interface__
    shape = tuple(int(s) for s in cai["shape"])
    dtype = np.dtype(cai["typestr"])
    strides = cai.get("strides")
    if strides is not None:
        want, step = [], dtype.itemsize
        for s in reversed(shape):
            want.append(step)
            step *= s
        if tuple(strides) != tuple(reversed(want)) and int(np.prod(shape)) > 1:
            raise ValueError("device array must be C-contiguous")
    return int(cai["data"][0] or 0), shape, dtype


PINNED_MIN = 1 << 15  # entries; smaller host arrays stay ordinary numpy arrays


class _PinnedBlock:
    """Owner of a page-locked host block; numpy arrays made from it keep it
    alive (it is their base) and the block returns to the library's cache when
    the last one goes away."""

    __slots__ = ("ptr", "n", "__weakref__")

    def __init__(self, n: int):
        self.ptr = 0
        self.n = n
        p = ctypes.c_void_p()
        check(lib().gp_host_alloc(ctypes.byref(p), n * 8))
        self.ptr = p.value or 0

    @property
    def __array_interface__(self):
        return {"shape": (self.n,), "typestr": "<f8", "data": (self.ptr, False), "version": 3}

    def __del__(self):
        if self.ptr:
            try:
                lib().gp_host_free(self.ptr)
            except Exception:
                pass
            self.ptr = 0


def host_zeros(n: int) -> np.ndarray:
    """A zeroed float64 host array; page-locked (pinned) when large and a CUDA
    device is present, so copies to and from the device run at the full link
    rate."""
    n = max(int(n), 0)
    if n >= PINNED_MIN and has_device():
        try:
            a = np.asarray(_PinnedBlock(n))
            a.fill(0.0)
            return a
        except Exception:
            pass
    return np.zeros(n, dtype=np.float64)


def ptr(a) -> int:
    """Device address of a DeviceArray or a torch tensor (0 for None or an
    empty array)."""
    if a is None:
        return 0
    if isinstance(a, DeviceArray):
        return a.ptr
    if hasattr(a, "data_ptr"):
        return int(a.data_ptr()) if a.numel() else 0
    v = device_view(a)
    return v[0] if v is not None else 0
