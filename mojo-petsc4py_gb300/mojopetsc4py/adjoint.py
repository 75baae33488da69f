"""Differentiable sparse solve: a torch.autograd.Function around the device
Krylov solve.

    x = sparse_solve(values, b, system)        # A(values) x = b

`values` holds the stored entries of a CSR matrix with a fixed pattern
(`SparseSystem`), `b` the right-hand side; both are FP64 CUDA tensors.  The
forward pass is the library's KSP solve (GMRES(30) + ILU(0) by default, as
the reference configures `KSP().setType("gmres")` with `PC.setType("ilu")`).
The hand-written backward pass runs the adjoint solve

    A^T lambda = dL/dx

and returns

    dL/db      = lambda
    dL/dA_ij   = -lambda_i x_j     on the stored nonzeros (gp_mat_outer_on_pattern)

In FP64 the adjoint solve is the transposed solve of the forward system
(KSPSolveTranspose, `gp_ksp_set_transpose`): the same Krylov method, every
multiply by A replaced by one by A^T (the matrix's cached transposed
pattern, the reference's MatMultTranspose, src/ported.mojo:408-431) and every
preconditioner apply by the true transposed apply of the forward
preconditioner (for ILU the solves with U^T and L^T of the same factor) --
no second matrix and no second factorisation.  SOR, which has no transposed
apply here, solves with the transposed matrix built on the device
(`gp_mat_transpose`, the reference's `Mat.transpose`,
python/mojopetsc4py/PETSc/Mat.py:555-563) and its own SOR.

With `precision="mixed"` both solves are the library's mixed-precision form
(`gp_mixed_solve`): FP32 FGMRES(restart) preconditioned with the ILU(0) factor
rounded to FP32, inside FP64 iterative refinement that stops on the true FP64
residual ||b - A x|| <= rtol ||b||.  The forward solve runs on A and the
adjoint solve on the device-built A^T with its own ILU(0), so the gradient has
the accuracy of two FP64 solves to rtol.

torch is plumbing here: tensors hold device memory, the autograd engine calls
backward; every kernel is the library's.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _device as dev
from ._lib import KspOptions, KspResult, PcOptions, check, lib

_KSP = {"cg": 2, "bcgs": 6, "gmres": 12, "fgmres": 40}
_PC = {"none": 0, "jacobi": 2, "sor": 4, "ilu": 5, "icc": 6}

REASON_NAMES = {2: "CONVERGED_RTOL", 3: "CONVERGED_ATOL", 4: "CONVERGED_ITS"}


class SolveError(RuntimeError):
    """The forward or adjoint Krylov solve did not converge."""


class _Solver:
    """One matrix handle with its PC and KSP handles."""

    def __init__(self, mat: int, ksp_type: str, pc_type: str, rtol: float, atol: float,
                 max_it: int, restart: int):
        self.mat = mat
        self.pc = None
        self.ksp = None
        self.ksp_type, self.pc_type = ksp_type, pc_type
        self.rtol, self.atol, self.max_it, self.restart = rtol, atol, max_it, restart
        self.its = 0
        self.reason = 0
        self.rnorm = 0.0
        self.ksp_t = None  # the transposed solve's KSP (its own captured graph)

    def _options(self):
        o = KspOptions()
        lib().gp_ksp_options_default(ctypes.byref(o))
        o.type = _KSP[self.ksp_type]
        o.rtol, o.atol = self.rtol, self.atol
        o.max_it = self.max_it
        o.restart = self.restart
        return o

    def setup(self, fresh_pattern: bool):
        st = dev.stream_ptr()
        if self.pc is None:
            h = ctypes.c_void_p()
            check(lib().gp_pc_create(ctypes.byref(h)))
            self.pc = h.value
            o = PcOptions()
            lib().gp_pc_options_default(ctypes.byref(o))
            o.type = _PC[self.pc_type]
            check(lib().gp_pc_set_options(self.pc, ctypes.byref(o)))
            fresh_pattern = True
        if fresh_pattern:
            check(lib().gp_pc_setup(self.pc, self.mat, st))
        else:
            check(lib().gp_pc_update_values(self.pc, st))
        if self.ksp is None:
            h = ctypes.c_void_p()
            check(lib().gp_ksp_create(ctypes.byref(h)))
            self.ksp = h.value
            check(lib().gp_ksp_set_options(self.ksp, ctypes.byref(self._options())))

    def solve(self, b, x, transpose: bool = False):
        """A x = b, or A^T x = b with `transpose` (same matrix, same
        preconditioner: gp_ksp_set_transpose)."""
        if transpose and self.ksp_t is None:
            h = ctypes.c_void_p()
            check(lib().gp_ksp_create(ctypes.byref(h)))
            self.ksp_t = h.value
            check(lib().gp_ksp_set_options(self.ksp_t, ctypes.byref(self._options())))
            check(lib().gp_ksp_set_transpose(self.ksp_t, 1))
        ksp = self.ksp_t if transpose else self.ksp
        # the solve graph is keyed on the vector addresses: solve between two
        # fixed buffers so one captured graph serves every call
        if getattr(self, "_bbuf", None) is None or self._bbuf.numel() != b.numel():
            self._bbuf = b.clone()
            self._xbuf = b.new_empty(b.shape)
        else:
            self._bbuf.copy_(b)
        res = KspResult()
        check(lib().gp_ksp_solve(ksp, self.mat, self.pc, dev.ptr(self._bbuf),
                                 dev.ptr(self._xbuf), ctypes.byref(res), None, 0,
                                 dev.stream_ptr()))
        x.copy_(self._xbuf)
        self.its, self.reason, self.rnorm = int(res.its), int(res.reason), float(res.rnorm)
        if self.reason < 0:
            raise SolveError(f"{self.ksp_type}+{self.pc_type} diverged: reason {self.reason} "
                             f"after {self.its} iterations (residual {self.rnorm:.3e})")

    def close(self):
        if self.ksp is not None:
            lib().gp_ksp_destroy(self.ksp)
        if self.ksp_t is not None:
            lib().gp_ksp_destroy(self.ksp_t)
        if self.pc is not None:
            lib().gp_pc_destroy(self.pc)
        self.ksp = self.ksp_t = self.pc = None


class _TransposeView:
    """Iteration statistics of a solver's last transposed solve."""

    def __init__(self, solver):
        self.its, self.reason, self.rnorm = solver.its, solver.reason, solver.rnorm

    def close(self):
        pass


class _MixedSolver:
    """One matrix handle with an ILU(0) PC and a mixed-precision solver
    handle; same interface as `_Solver`."""

    def __init__(self, mat: int, rtol: float, max_outer: int, restart: int,
                 inner_rtol: float = 1e-4, tri_sweeps: int = None, tri_block: int = None):
        self.mat = mat
        self.pc = None
        self.h = None
        self.ksp_type, self.pc_type = "mixed-fgmres", "ilu"
        self.rtol, self.max_outer, self.restart = rtol, max_outer, restart
        self.inner_rtol, self.tri_sweeps, self.tri_block = inner_rtol, tri_sweeps, tri_block
        self.its = 0         # inner FP32 iterations
        self.passes = 0      # FP64 refinement passes
        self.reason = 0
        self.rnorm = 0.0     # true relative residual

    def setup(self, fresh_pattern: bool):
        st = dev.stream_ptr()
        if self.pc is None:
            h = ctypes.c_void_p()
            check(lib().gp_pc_create(ctypes.byref(h)))
            self.pc = h.value
            o = PcOptions()
            lib().gp_pc_options_default(ctypes.byref(o))
            o.type = _PC["ilu"]
            check(lib().gp_pc_set_options(self.pc, ctypes.byref(o)))
            fresh_pattern = True
        if fresh_pattern:
            check(lib().gp_pc_setup(self.pc, self.mat, st))
        else:
            check(lib().gp_pc_update_values(self.pc, st))
        if self.h is None:
            h = ctypes.c_void_p()
            check(lib().gp_mixed_create(ctypes.byref(h)))
            self.h = h.value

    def solve(self, b, x):
        from .mixed import MixedOptions, MixedResult

        # the refinement pass graph is keyed on the vector addresses
        if getattr(self, "_bbuf", None) is None or self._bbuf.numel() != b.numel():
            self._bbuf = b.clone()
            self._xbuf = b.new_empty(b.shape)
        else:
            self._bbuf.copy_(b)
        o = MixedOptions()
        lib().gp_mixed_options_default(ctypes.byref(o))
        o.restart, o.max_outer = self.restart, self.max_outer
        if self.tri_sweeps is not None:
            o.tri_sweeps = self.tri_sweeps
        if self.tri_block is not None:
            o.tri_block = self.tri_block
        o.rtol, o.inner_rtol = self.rtol, self.inner_rtol
        res = MixedResult()
        check(lib().gp_mixed_solve(self.h, self.mat, self.pc, ctypes.byref(o),
                                   dev.ptr(self._bbuf), dev.ptr(self._xbuf), ctypes.byref(res),
                                   dev.stream_ptr()))
        x.copy_(self._xbuf)
        self.its, self.passes, self.rnorm = int(res.inner_its), int(res.passes), float(res.relres)
        self.reason = 2 if res.converged else -3
        if not res.converged:
            raise SolveError(f"mixed-precision solve stopped after {self.passes} passes "
                             f"({self.its} inner iterations) at relative residual "
                             f"{self.rnorm:.3e} > {self.rtol:.1e}")

    def close(self):
        if self.h is not None:
            lib().gp_mixed_destroy(self.h)
        if self.pc is not None:
            lib().gp_pc_destroy(self.pc)
        self.h = self.pc = None


class SparseSystem:
    """A x = b for a square CSR pattern that stays fixed while its values
    change: the forward solver on A and, built on first use, the adjoint
    solver on A^T."""

    def __init__(self, indptr, indices, ksp_type: str = "gmres", pc_type: str = "ilu",
                 rtol: float = 1e-10, atol: float = 1e-50, max_it: int = 10000,
                 restart: int = 30, precision: str = "fp64"):
        torch = dev.torch()
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
        if precision == "mixed" and pc_type != "ilu":
            raise NotImplementedError("the mixed-precision solve is preconditioned with ilu")
        self.indptr = np.ascontiguousarray(indptr, dtype=np.int64)
        self.indices = np.ascontiguousarray(indices, dtype=np.int64)
        self.n = len(self.indptr) - 1
        self.nnz = int(self.indptr[-1])
        if ksp_type not in _KSP or pc_type not in _PC:
            raise NotImplementedError(f"unsupported solver {ksp_type}+{pc_type}")
        zeros = np.zeros(max(self.nnz, 1))
        h = ctypes.c_void_p()
        check(lib().gp_mat_create(ctypes.byref(h), self.n, self.n, self.nnz,
                                  self.indptr.ctypes.data, self.indices.ctypes.data,
                                  zeros.ctypes.data))
        self._mat = h.value
        self._matT = None
        if precision == "mixed":
            self._make = lambda mat: _MixedSolver(mat, rtol, max(1, max_it // restart), restart)
        else:
            cfg = (ksp_type, pc_type, rtol, atol, max_it, restart)
            self._make = lambda mat: _Solver(mat, *cfg)
        self.precision = precision
        self.forward_solver = self._make(self._mat)
        self.adjoint_solver = None
        self._version = 0          # bumped by every set_values
        self._adjoint_version = -1
        self._fwd_version = -1
        self._torch = torch

    def __del__(self):
        try:
            self.forward_solver.close()
            if self.adjoint_solver is not None:
                self.adjoint_solver.close()
            if self._matT is not None:
                lib().gp_mat_destroy(self._matT)
            lib().gp_mat_destroy(self._mat)
        except Exception:
            pass

    # ------------------------------------------------------------ values
    def set_values(self, values) -> None:
        v = self._check(values, self.nnz, "values")
        check(lib().gp_mat_set_values(self._mat, dev.ptr(v) if self.nnz else None, 1,
                                      dev.stream_ptr()))
        self._version += 1

    def _check(self, t, n, name):
        torch = self._torch
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
            raise TypeError(f"{name} must be a CUDA tensor")
        if t.dtype != torch.float64 or t.numel() != n:
            raise ValueError(f"{name} must be float64 with {n} entries")
        return t.detach().contiguous()

    # ------------------------------------------------------------ solves
    def solve(self, b):
        """x with A x = b for the current values (device tensors)."""
        b = self._check(b, self.n, "b")
        s = self.forward_solver
        if self._fwd_version != self._version:
            s.setup(fresh_pattern=self._fwd_version < 0)
            self._fwd_version = self._version
        x = self._torch.empty_like(b)
        if self.n:
            s.solve(b, x)
        return x

    def solve_transpose(self, g):
        """lambda with A^T lambda = g for the current values."""
        g = self._check(g, self.n, "g")
        if self.precision == "fp64" and self.forward_solver.pc_type != "sor":
            # the forward system's transposed solve: same matrix, same factor
            s = self.forward_solver
            if self._fwd_version != self._version:
                s.setup(fresh_pattern=self._fwd_version < 0)
                self._fwd_version = self._version
            lam = self._torch.empty_like(g)
            if self.n:
                s.solve(g, lam, transpose=True)
            self.adjoint_solver = _TransposeView(s)
            return lam
        st = dev.stream_ptr()
        fresh = False
        if self._matT is None:
            h = ctypes.c_void_p()
            check(lib().gp_mat_transpose(self._mat, ctypes.byref(h), st))
            self._matT = h.value
            self.adjoint_solver = self._make(self._matT)
            fresh = True
        elif self._adjoint_version != self._version:
            check(lib().gp_mat_transpose_values(self._mat, self._matT, st))
        if fresh or self._adjoint_version != self._version:
            self.adjoint_solver.setup(fresh_pattern=fresh)
            self._adjoint_version = self._version
        lam = self._torch.empty_like(g)
        if self.n:
            self.adjoint_solver.solve(g, lam)
        return lam

    def value_gradient(self, lam, x):
        """dL/dA on the stored nonzeros: -lambda_i x_j."""
        out = self._torch.empty(max(self.nnz, 1), dtype=self._torch.float64,
                                device=lam.device)[: self.nnz]
        if self.nnz:
            check(lib().gp_mat_outer_on_pattern(self._mat, dev.ptr(lam), dev.ptr(x), -1.0,
                                                dev.ptr(out), dev.stream_ptr()))
        return out


def _function():
    torch = dev.torch()

    class SparseSolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, values, b, system):
            system.set_values(values)
            x = system.solve(b)
            ctx.system = system
            ctx.version = system._version
            ctx.save_for_backward(values, x)
            return x

        @staticmethod
        def backward(ctx, gx):
            values, x = ctx.saved_tensors
            system = ctx.system
            if system._version != ctx.version:  # values changed since forward
                system.set_values(values)
                ctx.version = system._version
            lam = system.solve_transpose(gx.contiguous())
            gvals = system.value_gradient(lam, x) if ctx.needs_input_grad[0] else None
            gb = lam if ctx.needs_input_grad[1] else None
            return gvals, gb, None

    return SparseSolve


_FN = None


def sparse_solve(values, b, system: SparseSystem):
    """x = A(values)^-1 b, differentiable in `values` and `b`."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(values, b, system)
