"""Sequential vectors, mirroring `petsc4py.PETSc.Vec` as the reference does
(python/mojopetsc4py/PETSc/Vec.py).

Storage lives in two places: a host float64 ndarray (what `getArray` returns)
and a device copy in HBM.  A flag records which side is current, as PETSc's
own CUDA vectors do: every kernel runs on the GPU and leaves the device copy
current; `getArray` brings the host array up to date (into the same ndarray
object every time) and, unless `readonly=True`, marks the host side as the
one that may now be modified.  Host-side edits (`setArray`, `setValues`,
item assignment) are uploaded before the next kernel.
"""

from __future__ import annotations

import ctypes

import numpy as np

from .. import _device as dev
from .._lib import check, lib

# which copy is current
_HOST, _DEVICE, _BOTH = 1, 2, 3

# gp_vec_map operation codes (include/gpetsc.h)
OP_COPY, OP_SET, OP_SCALE, OP_SHIFT, OP_AXPY, OP_AYPX, OP_AXPBY, OP_AXPBYPCZ = range(8)
OP_WAXPY, OP_PMULT, OP_PDIV, OP_PMIN, OP_PMAX, OP_PMAXABS, OP_RECIP, OP_EXP = range(8, 16)
OP_LOG, OP_SQRTABS, OP_ABS, OP_CHOP, OP_SWAP, OP_ZERO, OP_SCALESET, OP_DIVS = range(16, 24)
RED_DOT, RED_NORM2SQ, RED_ASUM, RED_SUM, RED_DOTNORM2, RED_NORMINF = range(6)


class VecType:
    """The vector type."""

    SEQ = "seq"
    STANDARD = "seq"
    MPI = "mpi"
    SHARED = "shared"
    NEST = "nest"
    CUDA = "seqcuda"


class NormType:
    """petscvec.h NormType."""

    NORM_1 = 0
    NORM_2 = 1
    NORM_FROBENIUS = 2
    NORM_INFINITY = 3
    NORM_1_AND_2 = 4
    N_1 = NORM_1
    NORM_MAX = NORM_INFINITY


def _f64(a, copy=False):
    if copy:
        return np.array(a, dtype=np.float64, order="C", copy=True)
    return np.ascontiguousarray(a, dtype=np.float64)


class Vec:
    """A sequential PETSc vector whose kernels run on the GPU."""

    Type = VecType

    def __init__(self):
        self._h = None
        self._d = None
        self._loc = _HOST
        self._bsize = 1

    # ---------------------------------------------------------- storage
    def _init_storage(self, arr: np.ndarray):
        self._h = arr
        self._d = None
        self._loc = _HOST

    def _check(self):
        if self._h is None:
            raise RuntimeError("Vec has not been created")
        return self._h

    def _size(self) -> int:
        return len(self._check())

    def _dptr(self) -> int:
        """Device pointer with the device copy current (for reading)."""
        n = self._size()
        if self._d is None:
            self._d = dev.DeviceArray(n)
            if self._loc == _DEVICE:
                self._loc = _HOST
        if self._loc == _HOST:
            dev.upload(self._d.ptr, self._h)
            self._loc = _BOTH
        return self._d.ptr

    def _wptr(self) -> int:
        """Device pointer for a kernel that writes: the device side becomes the
        only current copy."""
        p = self._dptr()
        self._loc = _DEVICE
        return p

    def _optr(self) -> int:
        """Device pointer for a kernel that overwrites every entry without
        reading it: no upload needed."""
        n = self._size()
        if self._d is None:
            self._d = dev.DeviceArray(n)
        self._loc = _DEVICE
        return self._d.ptr

    def _sync_host(self):
        if self._loc == _DEVICE:
            dev.download(self._h, self._d.ptr)
            self._loc = _BOTH

    # ---------------------------------------------------------- creation
    def create(self, comm=None) -> "Vec":
        self._h = None
        self._d = None
        self._bsize = 1
        return self

    def createSeq(self, size, bsize=None, comm=None) -> "Vec":
        n = int(size[0] if isinstance(size, (tuple, list)) else size)
        bs = 1 if bsize is None else int(bsize)
        if bs < 1:
            raise ValueError(f"invalid block size {bs}")
        if n % bs:
            raise ValueError(f"global size {n} not divisible by block size {bs}")
        self._init_storage(dev.host_zeros(n))
        self._bsize = bs
        return self

    def createWithArray(self, array, bsize=None, comm=None) -> "Vec":
        src = _f64(array)
        arr = dev.host_zeros(len(src))
        arr[:] = src
        bs = 1 if bsize is None else int(bsize)
        if len(arr) % bs:
            raise ValueError(
                f"array length {len(arr)} is not a multiple of the block size {bs}"
            )
        self._init_storage(arr)
        self._bsize = bs
        return self

    def duplicate(self, array=None) -> "Vec":
        out = Vec()
        out._bsize = self._bsize
        if array is None:
            out._init_storage(dev.host_zeros(self._size()))
        else:
            src = _f64(array)
            arr = dev.host_zeros(len(src))
            arr[:] = src
            if len(arr) != self._size():
                raise ValueError(f"incompatible array size: {len(arr)} != {self._size()}")
            out._init_storage(arr)
        return out

    def copy(self, result=None) -> "Vec":
        target = self.duplicate() if result is None else result
        self._peer(target)
        self._map(OP_COPY, target, x=self, write_only=True)
        return target

    def destroy(self) -> "Vec":
        self._h = None
        self._d = None
        return self

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    # ---------------------------------------------------------- accessors
    def getArray(self, readonly: bool = False) -> np.ndarray:
        """The local storage as an ndarray (the same object on every call),
        brought up to date with the device."""
        self._check()
        self._sync_host()
        if not readonly:
            self._loc = _HOST
        return self._h

    def setArray(self, array) -> None:
        """Copy `array` into the vector.  A large vector takes it straight to
        its device block (a host-to-device copy runs at the link rate from any
        host memory, while a copy into the page-locked host array first costs a
        host memcpy of the same size); the host array is brought up to date by
        the next getArray, as after any kernel that writes the vector."""
        cur = self._check()
        arr = _f64(array)
        if len(arr) != len(cur):
            raise ValueError(f"incompatible array size: {len(arr)} != {len(cur)}")
        if len(arr) >= dev.PINNED_MIN and dev.has_device():
            if self._d is None:
                self._d = dev.DeviceArray(len(arr))
            dev.upload(self._d.ptr, arr)
            self._loc = _DEVICE
            return
        cur[:] = arr
        self._loc = _HOST

    def placeArray(self, array) -> None:
        self.setArray(array)

    def getSize(self) -> int:
        return self._size()

    def getLocalSize(self) -> int:
        return self._size()

    def getSizes(self):
        n = self._size()
        return (n, n)

    def getBlockSize(self) -> int:
        return self._bsize

    def getOwnershipRange(self):
        return (0, self._size())

    def getType(self) -> str:
        return "seq"

    def getValue(self, index: int) -> float:
        return float(self.getArray(readonly=True)[index])

    def setValue(self, index: int, value: float) -> None:
        self.getArray()[index] = value

    def getValues(self, indices) -> np.ndarray:
        return self.getArray(readonly=True)[np.asarray(indices, dtype=np.int64)]

    def setValues(self, indices, values, addv=None) -> None:
        idx = np.asarray(indices, dtype=np.int64)
        val = _f64(values)
        arr = self.getArray()
        if addv is None:
            arr[idx] = val
        else:
            arr[idx] += val

    # ---------------------------------------------------------- kernels
    def _peer(self, *others: "Vec") -> None:
        n = self._size()
        for other in others:
            if other._size() != n:
                raise ValueError(f"incompatible sizes: {n} and {other._size()}")

    def _map(self, op, y: "Vec", x: "Vec" = None, w: "Vec" = None, alpha=0.0, beta=0.0,
             gamma=0.0, write_only=False):
        n = y._size()
        if n == 0:
            return
        xp = x._dptr() if x is not None else 0
        wp = w._dptr() if w is not None else 0
        yp = y._optr() if write_only else y._wptr()
        check(lib().gp_vec_map(op, n, yp, xp, wp, float(alpha), float(beta), float(gamma),
                               dev.stream_ptr()))

    def _reduce(self, op, other: "Vec" = None, nout=1):
        out = (ctypes.c_double * 2)()
        n = self._size()
        xp = self._dptr() if n else 0
        yp = other._dptr() if (other is not None and n) else 0
        check(lib().gp_vec_reduce(op, n, xp, yp, out, dev.stream_ptr()))
        return out[0] if nout == 1 else (out[0], out[1])

    # ---------------------------------------------------------- reductions
    def norm(self, norm_type=None):
        """NORM_2 (default), NORM_1, NORM_INFINITY, NORM_FROBENIUS, or the pair
        for NORM_1_AND_2 (src/ported.mojo:113-135)."""
        ntype = NormType.NORM_2 if norm_type is None else int(norm_type)
        n = self._size()
        if ntype in (NormType.NORM_2, NormType.NORM_FROBENIUS):
            return float(np.sqrt(self._reduce(RED_NORM2SQ))) if n else 0.0
        if ntype == NormType.NORM_1:
            return float(self._reduce(RED_ASUM)) if n else 0.0
        if ntype == NormType.NORM_INFINITY:
            return float(self._reduce(RED_NORMINF)) if n else 0.0
        if ntype == NormType.NORM_1_AND_2:
            if not n:
                return (0.0, 0.0)
            return (float(self._reduce(RED_ASUM)), float(np.sqrt(self._reduce(RED_NORM2SQ))))
        raise ValueError(f"unknown norm type {norm_type}")

    def normBegin(self, norm_type=None) -> None:
        return None

    def normEnd(self, norm_type=None):
        return self.norm(norm_type)

    def dot(self, other: "Vec") -> float:
        self._peer(other)
        return float(self._reduce(RED_DOT, other))

    def tDot(self, other: "Vec") -> float:
        """y^T x without the conjugate: the dot with the arguments swapped
        (src/ported.mojo:320-323)."""
        self._peer(other)
        return float(other._reduce(RED_DOT, self))

    def dotNorm2(self, other: "Vec"):
        """(self . other, ||self||^2) in one pass (src/ported.mojo:143-152)."""
        self._peer(other)
        d, q = self._reduce(RED_DOTNORM2, other, nout=2)
        return (float(d), float(q))

    def sum(self) -> float:
        return float(self._reduce(RED_SUM))

    def mean(self) -> float:
        return float(self._reduce(RED_SUM)) / float(self._size())

    def _minmax(self, is_max):
        idx = ctypes.c_int64(0)
        val = ctypes.c_double(0.0)
        n = self._size()
        check(lib().gp_vec_minmax(n, self._dptr() if n else 0, int(is_max), ctypes.byref(idx),
                                  ctypes.byref(val), dev.stream_ptr()))
        return (int(idx.value), float(val.value))

    def min(self):
        return self._minmax(False)

    def max(self):
        return self._minmax(True)

    def normalize(self) -> float:
        """Divide by the 2-norm when it is positive; return the norm."""
        z = self.norm()
        if z > 0.0:
            # VecNormalize divides (simdvec.normalize_inplace): x / z
            self._map(OP_DIVS, self, alpha=z)
        return z

    def maxPointwiseDivide(self, other: "Vec") -> float:
        self._peer(other)
        out = ctypes.c_double(0.0)
        n = self._size()
        check(lib().gp_vec_max_pointwise_divide(n, self._dptr() if n else 0,
                                                other._dptr() if n else 0,
                                                ctypes.byref(out), dev.stream_ptr()))
        return float(out.value)

    # ---------------------------------------------------------- elementwise
    def zeroEntries(self) -> None:
        self._map(OP_ZERO, self, write_only=True)

    def set(self, alpha) -> None:
        self._map(OP_SET, self, alpha=alpha, write_only=True)

    def scale(self, alpha) -> None:
        self._map(OP_SCALE, self, alpha=alpha)

    def shift(self, alpha) -> None:
        self._map(OP_SHIFT, self, alpha=alpha)

    def swap(self, other: "Vec") -> None:
        self._peer(other)
        n = self._size()
        if n:
            xp = other._wptr()
            check(lib().gp_vec_map(OP_SWAP, n, self._wptr(), xp, 0, 0.0, 0.0, 0.0,
                                   dev.stream_ptr()))

    def axpy(self, alpha, other: "Vec") -> None:
        """y = alpha*x + y."""
        self._peer(other)
        self._map(OP_AXPY, self, x=other, alpha=alpha)

    def aypx(self, alpha, other: "Vec") -> None:
        """y = x + alpha*y."""
        self._peer(other)
        self._map(OP_AYPX, self, x=other, alpha=alpha)

    def axpby(self, alpha, beta, other: "Vec") -> None:
        """y = alpha*x + beta*y."""
        self._peer(other)
        self._map(OP_AXPBY, self, x=other, alpha=alpha, beta=beta)

    def axpbypcz(self, alpha, beta, gamma, other, another) -> None:
        """z = alpha*x + beta*y + gamma*z."""
        self._peer(other, another)
        self._map(OP_AXPBYPCZ, self, x=other, w=another, alpha=alpha, beta=beta, gamma=gamma)

    def waxpy(self, alpha, other: "Vec", another: "Vec") -> None:
        """w = alpha*x + y."""
        self._peer(other, another)
        self._map(OP_WAXPY, self, x=other, w=another, alpha=alpha,
                  write_only=self is not other and self is not another)

    def maxpy(self, alphas, vecs) -> None:
        """y = y + sum_k alpha_k x_k."""
        alph = _f64(alphas)
        if len(alph) != len(vecs):
            raise ValueError("alphas and vecs must have the same length")
        for v in vecs:
            self._peer(v)
        n = self._size()
        if not n or not len(vecs):
            return
        ptrs = (ctypes.c_void_p * len(vecs))(*[v._dptr() for v in vecs])
        check(lib().gp_vec_maxpy(n, self._wptr(), len(vecs), alph.ctypes.data, ptrs,
                                 dev.stream_ptr()))

    def pointwiseMult(self, other: "Vec", another: "Vec") -> None:
        self._peer(other, another)
        self._map(OP_PMULT, self, x=other, w=another,
                  write_only=self is not other and self is not another)

    def pointwiseDivide(self, other: "Vec", another: "Vec") -> None:
        self._peer(other, another)
        self._map(OP_PDIV, self, x=other, w=another,
                  write_only=self is not other and self is not another)

    def pointwiseMin(self, other: "Vec", another: "Vec") -> None:
        self._peer(other, another)
        self._map(OP_PMIN, self, x=other, w=another,
                  write_only=self is not other and self is not another)

    def pointwiseMax(self, other: "Vec", another: "Vec") -> None:
        self._peer(other, another)
        self._map(OP_PMAX, self, x=other, w=another,
                  write_only=self is not other and self is not another)

    def pointwiseMaxAbs(self, other: "Vec", another: "Vec") -> None:
        self._peer(other, another)
        self._map(OP_PMAXABS, self, x=other, w=another,
                  write_only=self is not other and self is not another)

    def reciprocal(self) -> None:
        self._map(OP_RECIP, self)

    def exp(self) -> None:
        self._map(OP_EXP, self)

    def log(self) -> None:
        self._map(OP_LOG, self)

    def sqrtabs(self) -> None:
        self._map(OP_SQRTABS, self)

    def abs(self) -> None:
        self._map(OP_ABS, self)

    def conjugate(self) -> None:
        """The identity for real vectors."""
        return None

    def chop(self, tol) -> None:
        """Zero the entries with magnitude strictly below tol."""
        self._map(OP_CHOP, self, alpha=tol)

    # ---------------------------------------------------------- operators
    def __neg__(self):
        out = self.copy()
        out.scale(-1.0)
        return out

    def __pos__(self):
        return self.copy()

    def __abs__(self):
        out = self.copy()
        out.abs()
        return out

    def __add__(self, other):
        if not isinstance(other, Vec):
            return NotImplemented
        out = self.copy()
        out.axpy(1.0, other)
        return out

    __radd__ = __add__

    def __sub__(self, other):
        if not isinstance(other, Vec):
            return NotImplemented
        out = self.copy()
        out.axpy(-1.0, other)
        return out

    def __rsub__(self, other):
        if not isinstance(other, Vec):
            return NotImplemented
        return other - self

    def __mul__(self, other):
        if not isinstance(other, Vec):
            return NotImplemented
        out = self.duplicate()
        out.pointwiseMult(self, other)
        return out

    __rmul__ = __mul__

    def __truediv__(self, other):
        if not isinstance(other, Vec):
            return NotImplemented
        out = self.duplicate()
        out.pointwiseDivide(self, other)
        return out

    def __matmul__(self, other):
        return self.dot(other)

    def __getitem__(self, i):
        return self.getArray(readonly=True)[i]

    def __setitem__(self, i, v):
        self.getArray()[i] = v

    def __len__(self):
        return self._size()
