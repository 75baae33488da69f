"""Device memory and stream plumbing (PyTorch) for the PETSc classes.

Vectors keep their device copy in a torch tensor so the autograd wrapper can
hand it to torch without a copy; the CUDA work itself is all in libgpetsc.so.
"""

from __future__ import annotations

import numpy as np

_torch = None


def torch():
    global _torch
    if _torch is None:
        import torch as t

        if not t.cuda.is_available():
            raise RuntimeError(
                "mojopetsc4py (GB300 build) needs a CUDA device; torch sees none"
            )
        _torch = t
    return _torch


def stream_ptr() -> int:
    """The caller's current CUDA stream, as the void* the C ABI takes."""
    return int(torch().cuda.current_stream().cuda_stream)


def empty(n: int, dtype="float64"):
    t = torch()
    return t.empty(max(int(n), 0), dtype=getattr(t, dtype), device="cuda")


def from_host(a: np.ndarray):
    t = torch()
    return t.from_numpy(np.ascontiguousarray(a)).to("cuda", non_blocking=False)


PINNED_MIN = 1 << 15  # entries; smaller host arrays stay ordinary numpy arrays


def host_zeros(n: int) -> np.ndarray:
    """A zeroed float64 host array; page-locked (pinned) when large and a CUDA
    device is present, so copies to and from the device run at the full link
    rate.  The array keeps its pinned buffer alive."""
    n = max(int(n), 0)
    if n >= PINNED_MIN:
        try:
            t = torch()
            return t.zeros(n, dtype=t.float64, pin_memory=True).numpy()
        except Exception:
            pass
    return np.zeros(n, dtype=np.float64)


def ptr(tensor) -> int:
    return int(tensor.data_ptr()) if tensor is not None and tensor.numel() else 0
