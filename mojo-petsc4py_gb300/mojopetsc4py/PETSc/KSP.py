"""Krylov solvers, mirroring the reference's `KSP`
(python/mojopetsc4py/PETSc/KSP.py): cg, gmres, fgmres and bcgs with the same
setters, defaults, convergence test, residual history and converged reasons.

`solve(b, x)` runs the whole iteration on the GPU: the operator, the
preconditioner and the vectors stay in HBM, every scalar of the recurrence
stays in device memory, and the loop is one CUDA-graph launch (a WHILE node
whose body is one iteration).  It returns once the solve has finished, with
the iteration count, reason, residual norm and history read back.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from .. import _device as dev
from .._lib import KspOptions, KspResult, check, lib
from .Mat import Mat
from .PC import PC
from .Vec import Vec

DEFAULT_RTOL = 1e-5
DEFAULT_ATOL = 1e-50
DEFAULT_DTOL = 1.0e4
DEFAULT_MAX_IT = 1000
GMRES_DEFAULT_MAXK = 30


class KSPType:
    RICHARDSON = "richardson"
    CG = "cg"
    GMRES = "gmres"
    FGMRES = "fgmres"
    BCGS = "bcgs"
    MINRES = "minres"
    PREONLY = "preonly"


SUPPORTED = {KSPType.CG, KSPType.GMRES, KSPType.FGMRES, KSPType.BCGS}
_CODE = {KSPType.CG: 2, KSPType.BCGS: 6, KSPType.GMRES: 12, KSPType.FGMRES: 40}


class NormType_:
    NORM_DEFAULT = 0
    NORM_NONE = 1
    NORM_PRECONDITIONED = 2
    NORM_UNPRECONDITIONED = 3
    NORM_NATURAL = 4
    DEFAULT = 0
    NONE = 1
    NO = 1
    PRECONDITIONED = 2
    UNPRECONDITIONED = 3
    NATURAL = 4


class ConvergedReason:
    CONVERGED_ITERATING = 0
    ITERATING = 0
    CONVERGED_RTOL_NORMAL_EQUATIONS = 1
    CONVERGED_RTOL = 2
    CONVERGED_ATOL = 3
    CONVERGED_ITS = 4
    CONVERGED_NEG_CURVE = 5
    CONVERGED_STEP_LENGTH = 6
    CONVERGED_HAPPY_BREAKDOWN = 7
    CONVERGED_ATOL_NORMAL_EQUATIONS = 9
    DIVERGED_NULL = -2
    DIVERGED_ITS = -3
    DIVERGED_DTOL = -4
    DIVERGED_BREAKDOWN = -5
    DIVERGED_BREAKDOWN_BICG = -6
    DIVERGED_NONSYMMETRIC = -7
    DIVERGED_INDEFINITE_PC = -8
    DIVERGED_NANORINF = -9
    DIVERGED_INDEFINITE_MAT = -10
    DIVERGED_PC_FAILED = -11
    DIVERGED_INDEFINITE_PRECONDITIONER = -8
    DIVERGED_PCSETUP_FAILED = -11
    DIVERGED_MAX_IT = -3


class GMRESCGSRefinementType:
    REFINE_NEVER = 0
    REFINE_IFNEEDED = 1
    REFINE_ALWAYS = 2
    CGS_REFINE_NEVER = 0
    CGS_REFINE_IFNEEDED = 1
    CGS_REFINE_ALWAYS = 2


class GMRESOrthogonalizationType:
    CLASSICAL = 0
    MODIFIED = 1
    CGS = 0
    MGS = 1


class KSP:
    """A Krylov subspace solver for a sequential AIJ matrix, on the GPU."""

    Type = KSPType
    ConvergedReason = ConvergedReason
    NormType = NormType_
    GMRESCGSRefinementType = GMRESCGSRefinementType
    GMRESOrthogonalizationType = GMRESOrthogonalizationType

    def __init__(self):
        self._type = KSPType.GMRES
        self._amat = None
        self._pmat = None
        self._pc = PC()
        self._pc_side = 0
        self._normtype = 0
        self._rtol = DEFAULT_RTOL
        self._atol = DEFAULT_ATOL
        self._divtol = DEFAULT_DTOL
        self._max_it = DEFAULT_MAX_IT
        self._min_it = 0
        self._chknorm = -1
        self._convmaxits = 0
        self._guess_zero = 1
        self._restart = GMRES_DEFAULT_MAXK
        self._haptol = 1.0e-30
        self._breakdowntol = 0.1
        self._orthog = 0
        self._cgstype = 0
        self._its = 0
        self._rnorm = 0.0
        self._reason = 0
        self._history = None
        self._histlen = 0
        self._histreset = False
        self._rhs = None
        self._sol = None
        self._setupcalled = False
        self._gp = None
        self._launch_form = -1

    def __del__(self):
        h = getattr(self, "_gp", None)
        if h is not None:
            try:
                lib().gp_ksp_destroy(h)
            except Exception:
                pass

    # ---------------------------------------------------------- lifecycle
    def create(self, comm=None) -> "KSP":
        return self

    def destroy(self) -> "KSP":
        self._history = None
        return self

    def setType(self, ksp_type) -> None:
        if isinstance(ksp_type, int):
            raise TypeError("expected a Krylov type name")
        if ksp_type not in SUPPORTED:
            raise NotImplementedError(
                f"KSP type {ksp_type!r} is not covered by mojopetsc4py"
                f" ({sorted(SUPPORTED)} are)"
            )
        self._type = ksp_type
        self._setupcalled = False

    def getType(self) -> str:
        return self._type

    def setOperators(self, A: Mat = None, P: Mat = None) -> None:
        self._amat = A
        self._pmat = A if P is None else P
        self._pc.setOperators(self._amat, self._pmat)
        self._setupcalled = False

    def getOperators(self):
        return (self._amat, self._pmat)

    def setPC(self, pc: PC) -> None:
        self._pc = pc
        if self._pmat is not None:
            self._pc.setOperators(self._amat, self._pmat)
        self._setupcalled = False

    def getPC(self) -> PC:
        return self._pc

    def setPCSide(self, side) -> None:
        self._pc_side = int(side)

    def getPCSide(self):
        return self._pc_side

    def setNormType(self, normtype) -> None:
        self._normtype = int(normtype)

    def getNormType(self):
        return self._normtype

    def setTolerances(self, rtol=None, atol=None, divtol=None, max_it=None) -> None:
        """Setting max_it also makes reaching it report CONVERGED_ITS, as the
        reference does (python/mojopetsc4py/PETSc/KSP.py:212-225)."""
        if rtol is not None:
            self._rtol = float(rtol)
        if atol is not None:
            self._atol = float(atol)
        if divtol is not None:
            self._divtol = float(divtol)
        if max_it is not None:
            self._max_it = int(max_it)
            self._convmaxits = 1

    def getTolerances(self):
        return (self._rtol, self._atol, self._divtol, self._max_it)

    def setMinimumIterations(self, min_it) -> None:
        self._min_it = int(min_it)

    def getMinimumIterations(self) -> int:
        return self._min_it

    def setCheckNorm(self, flag) -> None:
        self._chknorm = int(flag)

    def setInitialGuessNonzero(self, flag) -> None:
        self._guess_zero = 0 if flag else 1

    def getInitialGuessNonzero(self) -> bool:
        return not self._guess_zero

    def setGMRESRestart(self, restart) -> None:
        self._restart = int(restart)
        self._setupcalled = False

    def setGMRESHapTol(self, haptol) -> None:
        self._haptol = float(haptol)

    def setGMRESBreakdownTolerance(self, tol) -> None:
        self._breakdowntol = float(tol)

    def setGMRESOrthogonalization(self, orthog) -> None:
        self._orthog = int(orthog)

    def setGMRESCGSRefinementType(self, cgstype) -> None:
        self._cgstype = int(cgstype)

    def setConvergenceHistory(self, length=None, reset: bool = False) -> None:
        size = 10000 if length is None or length is True else int(length)
        if size < 0:
            size = 10000
        self._histlen = size
        self._histreset = bool(reset)
        self._history = np.zeros(size, dtype=np.float64)

    def getConvergenceHistory(self) -> np.ndarray:
        if self._history is None:
            return np.zeros(0, dtype=np.float64)
        return self._history

    def getIterationNumber(self) -> int:
        return self._its

    def getResidualNorm(self) -> float:
        return self._rnorm

    def getConvergedReason(self):
        return self._reason

    def getRhs(self) -> Vec:
        return self._rhs

    def getSolution(self) -> Vec:
        return self._sol

    def setUp(self) -> None:
        if self._amat is None:
            raise RuntimeError("KSP.setOperators() has not been called")
        self._pc.setUp()
        self._setupcalled = True

    # ---------------------------------------------------------- solve
    def _resolve_normtype(self):
        """NORM_DEFAULT resolves to NORM_PRECONDITIONED for every covered type."""
        if self._normtype == NormType_.NORM_DEFAULT:
            self._normtype = NormType_.NORM_PRECONDITIONED

    def _rhs_norm(self, b: Vec, transpose: bool = False) -> float:
        """KSPConvergedDefault's right-hand-side norm for a nonzero guess
        (the reference computes it in Python, KSP.py:496-507; here the
        preconditioner apply and the norm run on the GPU)."""
        if self._normtype == NormType_.NORM_NONE:
            return 0.0
        if self._normtype == NormType_.UNPRECONDITIONED or self._pc_side == 1:
            return float(b.norm())
        z = b.duplicate()
        if transpose:
            self._pc._apply_transpose_exact(b, z)
        else:
            self._pc.apply(b, z)
        if self._normtype == NormType_.PRECONDITIONED:
            return float(z.norm())
        return math.sqrt(abs(z.dot(b)))

    def _options(self, rhs_norm: float) -> KspOptions:
        o = KspOptions()
        lib().gp_ksp_options_default(ctypes.byref(o))
        o.type = _CODE[self._type]
        o.normtype = int(self._normtype)
        o.pc_side = int(self._pc_side)
        o.guess_zero = int(self._guess_zero)
        o.min_it = int(self._min_it)
        o.chknorm = int(self._chknorm)
        o.convmaxits = int(self._convmaxits)
        o.max_it = int(self._max_it)
        o.restart = int(self._restart)
        o.orthog = int(self._orthog)
        o.cgstype = int(self._cgstype)
        o.seed_rhs = 0 if self._guess_zero else 1
        o.rtol, o.atol, o.divtol = self._rtol, self._atol, self._divtol
        o.haptol, o.breakdowntol = self._haptol, self._breakdowntol
        o.rhs_norm = float(rhs_norm)
        return o

    def solve(self, b: Vec, x: Vec) -> None:
        """Solve A x = b on the GPU; with the default zero initial guess the
        contents of x on entry are ignored."""
        self._solve(b, x, False)

    def solveTranspose(self, b: Vec, x: Vec) -> None:
        """Solve A^T x = b with the same operator and preconditioner: every
        multiply by A becomes one by A^T and every preconditioner apply the
        true transposed one (for ILU, the triangular solves with U^T and L^T
        of the same factor).  petsc4py's KSP.solveTranspose; the reference
        has no transposed solve."""
        self._solve(b, x, True)

    def _solve(self, b: Vec, x: Vec, transpose: bool) -> None:
        if self._amat is None:
            raise RuntimeError("KSP.setOperators() has not been called")
        A = self._amat
        A._materialize()
        n = A._nrows
        if A._nrows != A._ncols:
            raise ValueError("the solver matrix must be square")
        if b._size() != n or x._size() != n:
            raise ValueError(f"incompatible vector size: {n} is needed for both operands")
        if b is x:
            raise ValueError("x may not alias b")
        if not self._setupcalled:
            self.setUp()
        self._pc.setUp()
        self._rhs, self._sol = b, x
        self._resolve_normtype()
        rhs = 0.0 if self._guess_zero else self._rhs_norm(b, transpose)
        if self._gp is None:
            h = ctypes.c_void_p()
            check(lib().gp_ksp_create(ctypes.byref(h)))
            self._gp = h.value
        check(lib().gp_ksp_set_launch_form(self._gp, self._launch_form))
        check(lib().gp_ksp_set_transpose(self._gp, 1 if transpose else 0))
        opts = self._options(rhs)
        check(lib().gp_ksp_set_options(self._gp, ctypes.byref(opts)))
        hist = np.zeros(max(self._histlen, 0), dtype=np.float64)
        res = KspResult()
        bp = b._dptr() if n else 0
        # a zero guess ignores x on entry (the solver zeroes it): no upload
        xp = (x._optr() if self._guess_zero else x._wptr()) if n else 0
        check(lib().gp_ksp_solve(self._gp, A._device(), self._pc._handle(), bp, xp,
                                 ctypes.byref(res), hist.ctypes.data if len(hist) else None,
                                 len(hist), dev.stream_ptr()))
        self._its = int(res.its)
        self._reason = int(res.reason)
        self._rnorm = float(res.rnorm)
        self._history = hist

    def setLaunchForm(self, form: str = "graph"):
        """Extension (no counterpart in the reference): "graph" runs each
        solve as one captured CUDA graph; "host" launches the same kernels
        one by one from a host loop, so a profiler lists each of them;
        "default" follows GPETSC_KSP_GRAPH.  Results are identical."""
        forms = {"default": -1, "graph": 0, "host": 1}
        if form not in forms:
            raise ValueError(f"launch form must be one of {sorted(forms)}")
        self._launch_form = forms[form]

    def getLaunchStats(self):
        """(loop trips, kernels outside the loop, kernels per trip) of the last
        solve; kernels launched = outside + trips * per_trip."""
        t, a, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().gp_ksp_stats(self._gp, ctypes.byref(t), ctypes.byref(a), ctypes.byref(b)))
        return (t.value, a.value, b.value)
