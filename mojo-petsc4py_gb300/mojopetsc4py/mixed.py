"""Mixed precision solve: FP32 inner FGMRES(restart) + ILU(0) inside FP64
iterative refinement, to rtol on the true FP64 residual (include/gpetsc.h,
gp_mixed_*).

    solver = MixedSolver(A)                 # A: an assembled PETSc.Mat
    info = solver.solve(b, x, rtol=1e-10)   # b, x: PETSc.Vec

The ILU(0) factor is the plain path's (PC "ilu", same symbolic and numeric
phase), rounded to FP32; each triangle is applied with `tri_sweeps` passes:
point-Jacobi passes (`tri_block=0`) or block passes that solve runs of
`tri_block` consecutive rows exactly and couple the runs through the previous
pass (`tri_block=-1` picks the run length); `tri_sweeps=0` uses the exact
level-scheduled FP64 sweeps.
"""
from __future__ import annotations

import ctypes

from . import _device as dev
from ._lib import check, lib
from .PETSc import PC


class MixedOptions(ctypes.Structure):
    _fields_ = [("restart", ctypes.c_int32), ("max_outer", ctypes.c_int32),
                ("tri_sweeps", ctypes.c_int32), ("tri_block", ctypes.c_int32),
                ("rtol", ctypes.c_double), ("inner_rtol", ctypes.c_double)]


class MixedResult(ctypes.Structure):
    _fields_ = [("passes", ctypes.c_int32), ("inner_its", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("relres", ctypes.c_double)]


class MixedSolver:
    """`ordering="multicolor"` factors the inner ILU in a greedy multicolour
    ordering of the rows (a library extension; the reference has natural and
    RCM): every triangle then has one dependency level per colour, and
    `tri_sweeps` equal to the number of colours (two for 5- and 7-point
    stencils) applies it exactly with bandwidth-bound passes."""

    def __init__(self, A, levels: int = 0, ordering: str = "natural"):
        if ordering not in ("natural", "multicolor"):
            raise ValueError(f"ordering must be 'natural' or 'multicolor', not {ordering!r}")
        self.A = A
        self.pc = PC().create()
        self.pc.setType("ilu")
        if levels:
            self.pc.setFactorLevels(levels)
        self.pc._multicolor = ordering == "multicolor"
        self.pc.setOperators(A)
        h = ctypes.c_void_p()
        check(lib().gp_mixed_create(ctypes.byref(h)))
        self._h = h.value

    def __del__(self):
        try:
            lib().gp_mixed_destroy(self._h)
        except Exception:
            pass

    def solve(self, b, x, rtol: float = 1e-10, restart: int = 30, inner_rtol: float = 1e-4,
              tri_sweeps: int = None, max_outer: int = 200, tri_block: int = None):
        """x = A^-1 b with ||b - A x|| <= rtol ||b||; returns a dict with the
        passes, inner iterations, convergence flag and final relative
        residual."""
        A = self.A
        A._materialize()
        n = A._nrows
        if b._size() != n or x._size() != n:
            raise ValueError(f"incompatible vector size: {n} is needed for both operands")
        if b is x:
            raise ValueError("x may not alias b")
        self.pc.setUp()
        o = MixedOptions()
        lib().gp_mixed_options_default(ctypes.byref(o))
        o.restart, o.max_outer = int(restart), int(max_outer)
        if tri_sweeps is not None:
            o.tri_sweeps = int(tri_sweeps)
        if tri_block is not None:
            o.tri_block = int(tri_block)
        o.rtol, o.inner_rtol = float(rtol), float(inner_rtol)
        res = MixedResult()
        bp = b._dptr() if n else 0
        xp = x._optr() if n else 0
        check(lib().gp_mixed_solve(self._h, A._device(), self.pc._handle(), ctypes.byref(o),
                                   bp, xp, ctypes.byref(res), dev.stream_ptr()))
        return {"passes": res.passes, "inner_its": res.inner_its,
                "converged": bool(res.converged), "relres": res.relres}
