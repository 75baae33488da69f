"""Preconditioners, mirroring the reference's `PC`
(python/mojopetsc4py/PETSc/PC.py): types none, jacobi, sor, ilu and icc with
the same options, defaults and errors.

`setUp` builds the preconditioner for the operator on the GPU: the Jacobi
diagonals, the SOR diagonal, or the ILU/IC factor (symbolic pattern on the
host, numeric factorisation on the device).  `apply` runs the device kernels:
a pointwise multiply for Jacobi, and level-ordered sync-free triangular
sweeps for SOR, ILU and IC.
"""

from __future__ import annotations

import ctypes

import numpy as np

from .. import _device as dev
from .._lib import PcOptions, check, lib
from .Mat import Mat, MatOrderingType, from_dense
from .Vec import Vec

_NONE, _JACOBI, _SOR, _ILU, _ICC = 0, 2, 4, 5, 6

SOR_ZERO_INITIAL_GUESS = 16
SOR_FORWARD_SWEEP = 1
SOR_BACKWARD_SWEEP = 2
SOR_LOCAL_FORWARD_SWEEP = 4
SOR_LOCAL_BACKWARD_SWEEP = 8
SOR_LOCAL_SYMMETRIC_SWEEP = 12
SOR_EISENSTAT = 32
SOR_APPLY_UPPER = 64
SOR_APPLY_LOWER = 128

PC_JACOBI_DIAGONAL = 0
PC_JACOBI_ROWMAX = 1
PC_JACOBI_ROWL1 = 2
PC_JACOBI_ROWSUM = 3


class PCType:
    NONE = "none"
    JACOBI = "jacobi"
    SOR = "sor"
    LU = "lu"
    SHELL = "shell"
    BJACOBI = "bjacobi"
    ILU = "ilu"
    ICC = "icc"
    ASM = "asm"
    GASM = "gasm"
    KSP = "ksp"
    CHOLESKY = "cholesky"
    PYTHON = "python"
    MAT = "mat"
    FIELDSPLIT = "fieldsplit"
    LSC = "lsc"
    GAMG = "gamg"
    BDDC = "bddc"
    DEFLATION = "deflation"
    HPDDM = "hpddm"


SUPPORTED = {PCType.NONE, PCType.JACOBI, PCType.SOR, PCType.ILU, PCType.ICC}
_CODE = {PCType.NONE: _NONE, PCType.JACOBI: _JACOBI, PCType.SOR: _SOR, PCType.ILU: _ILU,
         PCType.ICC: _ICC}


class Side:
    LEFT = 0
    RIGHT = 1
    SYMMETRIC = 2
    DEFAULT = 0
    L = 0
    R = 1
    S = 2


class FailedReason:
    NOERROR = 0
    FACTOR_NUMERIC_ZEROPIVOT = 1
    FACTOR_NUMERIC_SINGULAR = 2
    FACTOR_INF_OR_NAN = 3
    FACTOR_OTHER = 4
    OUT_OF_MEMORY = 5
    SETUP_ERROR = 6
    SETUP_FAILED = 7
    PROBLEM_TOO_SMALL = 8


class PC:
    """A preconditioner for a sequential AIJ matrix, applied on the GPU."""

    Type = PCType
    Side = Side
    FailedReason = FailedReason

    def __init__(self):
        self._type = PCType.NONE
        self._amat = None
        self._pmat = None
        self._setupcalled = False
        self._use_amat = False
        self._reuse = False
        self._failed_reason = FailedReason.NOERROR
        self._levels = 0
        self._shift = 0.0
        self._zeropivot = 100.0
        self._shift_type = "none"
        self._ordering = MatOrderingType.NATURAL
        self._diagonal_fill = False
        self._sor_omega = 1.0
        self._sor_fshift = 0.0
        self._sor_its = 1
        self._sor_lits = 1
        self._sor_sym = "symmetric"
        self._fix_diag = True
        self._use_abs = False
        self._jacobi_type = PC_JACOBI_DIAGONAL
        self._rowl1_scale = 1.0
        self._gp = None
        self._gp_key = None
        self._exact_transpose = False

    def __del__(self):
        h = getattr(self, "_gp", None)
        if h is not None:
            try:
                lib().gp_pc_destroy(h)
            except Exception:
                pass

    # ---------------------------------------------------------- lifecycle
    def create(self, comm=None) -> "PC":
        return self

    def destroy(self) -> "PC":
        self._reset_factor()
        return self

    def setType(self, pc_type) -> None:
        if isinstance(pc_type, int):
            raise TypeError("expected a preconditioner type name")
        if pc_type not in SUPPORTED:
            raise NotImplementedError(f"PC type {pc_type!r} is not covered by mojopetsc4py")
        self._type = pc_type
        self._reset_factor()

    def getType(self) -> str:
        return self._type

    def setOperators(self, A: Mat = None, P: Mat = None) -> None:
        self._amat = A
        self._pmat = A if P is None else P
        self._reset_factor()

    def getOperators(self):
        return (self._amat, self._pmat)

    def setUseAmat(self, flag: bool) -> None:
        self._use_amat = bool(flag)

    def getUseAmat(self) -> bool:
        return self._use_amat

    def setReusePreconditioner(self, flag: bool) -> None:
        self._reuse = bool(flag)

    def setFailedReason(self, reason) -> None:
        self._failed_reason = reason

    def getFailedReason(self):
        return self._failed_reason

    def reset(self) -> None:
        self._reset_factor()

    def _reset_factor(self):
        self._setupcalled = False
        self._gp_key = None

    # ---------------------------------------------------------- options
    def setFactorLevels(self, levels) -> None:
        self._levels = int(levels)
        self._setupcalled = False

    def setFactorShift(self, shift_type, amount=None) -> None:
        """Only shift type `none` (the default, no pivot retry) is available,
        as in the reference."""
        name = str(shift_type)
        if name not in ("none", "positive_definite", "nonzero"):
            raise ValueError(f"unknown shift type: {name}")
        if name != "none":
            raise NotImplementedError(
                f"factor shift {name!r} is not covered by mojopetsc4py; only 'none'"
                " reproduces the reference factor"
            )
        self._shift_type = name
        if amount is not None:
            self._shift = float(amount)
        self._setupcalled = False

    def setFactorPivot(self, flag) -> None:
        """Only "no pivot check" (0 or False) is available, as in the reference."""
        tol = float(flag) if not isinstance(flag, bool) else (100.0 if flag else 0.0)
        if tol != 0.0:
            raise NotImplementedError(
                "a nonzero factor pivot tolerance is not covered by mojopetsc4py"
            )
        self._zeropivot = 0.0
        self._diagonal_fill = bool(flag)
        self._setupcalled = False

    def setFactorOrdering(self, ordering) -> None:
        if ordering not in (MatOrderingType.NATURAL, MatOrderingType.RCM):
            raise NotImplementedError(
                f"matrix ordering {ordering!r} is not covered by mojopetsc4py"
                " (natural and rcm are)"
            )
        self._ordering = ordering
        self._setupcalled = False

    def setFactorReorderForNonzeroDiagonal(self) -> None:
        self._diagonal_fill = True
        self._setupcalled = False

    def setSORSymmetric(self, flag) -> None:
        self._sor_sym = "symmetric" if flag else "forward"
        self._setupcalled = False

    def setSOROmega(self, omega) -> None:
        self._sor_omega = float(omega)
        self._setupcalled = False

    def setSORIterations(self, its) -> None:
        self._sor_its = int(its)
        self._setupcalled = False

    def setSORShift(self, fshift) -> None:
        self._sor_fshift = float(fshift)
        self._setupcalled = False

    def setJacobiType(self, jtype) -> None:
        self._jacobi_type = int(jtype)
        self._setupcalled = False

    def setJacobiUseAbs(self, flag) -> None:
        self._use_abs = bool(flag)
        self._setupcalled = False

    def setJacobiFixDiagonal(self, flag) -> None:
        self._fix_diag = bool(flag)
        self._setupcalled = False

    def setJacobiRowl1Scale(self, scale) -> None:
        self._rowl1_scale = float(scale)
        self._setupcalled = False

    def setFactorMatrixType(self, mtype) -> None:
        """Only seqaij is covered; accepted and ignored."""

    def setSPAIVerbose(self, level) -> None:
        raise NotImplementedError("spai is not covered by mojopetsc4py")

    # ---------------------------------------------------------- setup
    def _sor_flag(self) -> int:
        sweep = SOR_LOCAL_SYMMETRIC_SWEEP if self._sor_sym == "symmetric" else SOR_FORWARD_SWEEP
        return sweep | SOR_ZERO_INITIAL_GUESS

    def _options(self) -> PcOptions:
        o = PcOptions()
        lib().gp_pc_options_default(ctypes.byref(o))
        o.type = _CODE[self._type]
        o.jacobi_type = int(self._jacobi_type)
        o.use_abs = int(self._use_abs)
        o.fix_diag = int(self._fix_diag)
        o.rowl1_scale = float(self._rowl1_scale)
        o.omega = float(self._sor_omega)
        o.fshift = float(self._sor_fshift)
        o.sor_flag = self._sor_flag()
        o.levels = int(self._levels)
        o.ordering = 1 if self._ordering == MatOrderingType.RCM else 0
        if getattr(self, "_multicolor", False):
            o.ordering = 2
        return o

    def setUp(self) -> "PC":
        """Build the preconditioner for the operator on the GPU."""
        pmat = self._pmat
        if pmat is None:
            raise RuntimeError("PCSetOperators() has not been called")
        n = pmat._nrows
        if n != pmat._ncols:
            raise ValueError("the preconditioner matrix must be square")
        handle = pmat._device()
        key = (handle, pmat._pver)
        if self._setupcalled and self._gp is not None and self._gp_key == key:
            return self
        if self._gp is None:
            h = ctypes.c_void_p()
            check(lib().gp_pc_create(ctypes.byref(h)))
            self._gp = h.value
        opts = self._options()
        check(lib().gp_pc_set_options(self._gp, ctypes.byref(opts)))
        check(lib().gp_pc_setup(self._gp, handle, dev.stream_ptr()))
        self._gp_key = key
        self._setupcalled = True
        return self

    def _handle(self):
        self.setUp()
        return self._gp

    # ---------------------------------------------------------- apply
    def _check_pair(self, x: Vec, y: Vec):
        n = self._pmat._nrows
        if x._size() != n or y._size() != n:
            raise ValueError(f"incompatible vector size: {n} is needed for both operands")
        if x is y:
            raise ValueError("y may not alias x in a preconditioner apply")

    def apply(self, x: Vec, y: Vec) -> None:
        """y = M^-1 x."""
        self.setUp()
        self._check_pair(x, y)
        if self._pmat._nrows:
            check(lib().gp_pc_apply(self._gp, x._dptr(), y._optr(), dev.stream_ptr()))

    def applyTranspose(self, x: Vec, y: Vec) -> None:
        """The reference's applyTranspose is `apply` for every type
        (python/mojopetsc4py/PETSc/PC.py:635-642), and so is this one by
        default.  After `setUseExactTranspose(True)` it applies the true
        transpose M^-T (for ILU the solves with U^T and L^T of the factor),
        as upstream PETSc's PCApplyTranspose does."""
        if self._exact_transpose:
            self._apply_transpose_exact(x, y)
        else:
            self.apply(x, y)

    def setUseExactTranspose(self, flag: bool = True) -> None:
        """Extension (no counterpart in the reference): make applyTranspose
        the true transposed apply instead of the reference's plain apply."""
        self._exact_transpose = bool(flag)

    def _apply_transpose_exact(self, x: Vec, y: Vec) -> None:
        self.setUp()
        self._check_pair(x, y)
        if self._pmat._nrows:
            check(lib().gp_pc_apply_transpose(self._gp, x._dptr(), y._optr(),
                                              dev.stream_ptr()))

    def applySymmetricLeft(self, x: Vec, y: Vec) -> None:
        self.setUp()
        self._check_pair(x, y)
        if self._pmat._nrows:
            check(lib().gp_pc_apply_symmetric(self._gp, x._dptr(), y._optr(),
                                              dev.stream_ptr()))

    def applySymmetricRight(self, x: Vec, y: Vec) -> None:
        self.applySymmetricLeft(x, y)

    # ---------------------------------------------------------- factor
    def _factor_arrays(self):
        self.setUp()
        n = ctypes.c_int64()
        ns = ctypes.c_int64()
        check(lib().gp_pc_factor_info(self._gp, ctypes.byref(n), ctypes.byref(ns)))
        n, ns = n.value, ns.value
        bi = np.zeros(n + 1, dtype=np.int64)
        bj = np.zeros(max(ns, 1), dtype=np.int64)
        ba = np.zeros(max(ns, 1), dtype=np.float64)
        bdiag = np.zeros(n + 1, dtype=np.int64)
        perm = np.zeros(max(n, 1), dtype=np.int64)
        check(lib().gp_pc_factor_get(self._gp, bi.ctypes.data, bj.ctypes.data, ba.ctypes.data,
                                     bdiag.ctypes.data, perm.ctypes.data))
        return {"bi": bi, "bj": bj, "ba": ba, "bdiag": bdiag, "r": perm[:n], "c": perm[:n]}

    def getFactorMatrix(self) -> Mat:
        """The operator whose solve `apply` performs: L U for ILU, U^T D U for
        IC, as a CSR matrix in the caller's ordering."""
        if self._type not in (PCType.ILU, PCType.ICC):
            raise RuntimeError(f"PC type {self._type} has no factor matrix")
        f = self._factor_arrays()
        if self._type == PCType.ILU:
            return _ilu_product(f)
        return _icc_product(f)


def _ilu_product(f) -> Mat:
    """Dense L U from the ILU factor layout: L rows bi[i]..bi[i+1] (unit
    diagonal), U row i at bdiag[i+1]+1 .. bdiag[i]-1 with the inverted
    diagonal at bdiag[i]."""
    bi, bj, ba, bdiag, r = f["bi"], f["bj"], f["ba"], f["bdiag"], f["r"]
    n = len(bi) - 1
    L = np.eye(n)
    U = np.zeros((n, n))
    for i in range(n):
        for j in range(int(bi[i]), int(bi[i + 1])):
            L[int(r[i]), int(r[int(bj[j])])] = ba[j]
        for j in range(int(bdiag[i + 1]) + 1, int(bdiag[i])):
            U[int(r[i]), int(r[int(bj[j])])] = ba[j]
        U[int(r[i]), int(r[i])] = 1.0 / ba[int(bdiag[i])]
    return from_dense(L @ U)


def _icc_product(f) -> Mat:
    """Dense U^T D U from the IC layout: row i holds -U(i, j) for its strict
    upper columns, then 1/d_i in the diagonal slot bdiag[i]."""
    bi, bj, ba, bdiag, r = f["bi"], f["bj"], f["ba"], f["bdiag"], f["r"]
    n = len(bi) - 1
    unit = np.zeros((n, n))
    d = np.zeros(n)
    for i in range(n):
        row = int(r[i])
        unit[row, row] = 1.0
        for j in range(int(bi[i]), int(bdiag[i])):
            unit[int(r[int(bj[j])]), row] = -ba[j]
        inv = ba[int(bdiag[i])]
        d[row] = 1.0 / inv if inv != 0.0 else 0.0
    return from_dense((unit * d) @ unit.T)
