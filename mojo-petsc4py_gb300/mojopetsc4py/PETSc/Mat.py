"""Sequential AIJ (CSR) matrices, mirroring the reference's `Mat`
(python/mojopetsc4py/PETSc/Mat.py).

The host arrays are the reference's: int64 row starts, column indices
ascending within a row, float64 values.  Entries set after an assembly are
kept pending and folded into CSR on demand with the reference's semantics
(Mat.py:383-413, 434-439: per (row, col), INSERT sets and ADD adds, in call
order, from 0.0).  Blocks of entries (`setValues` with many indices) are
logged as arrays and large logs are folded on the GPU (gp_coo_assemble: a
stable radix sort and one fold per entry); `from_dense` and `transpose` also
run on the GPU for large matrices.  The multiply, the transposed multiply
and the diagonal run on the GPU against a device mirror (int32 indices) that
is created on first use and refreshed when the pattern or the values change.
"""

from __future__ import annotations

import ctypes

import numpy as np

from .. import _device as dev
from .._lib import check, lib
from .Vec import Vec


# logs of at least this many entries are folded on the GPU (smaller ones on
# the host, where a device round trip would cost more than the fold)
DEVICE_ASSEMBLY_MIN = 1 << 15
# setValues blocks of at least this many entries are logged as arrays (smaller
# ones go entry by entry, as in the reference)
BLOCK_LOG_MIN = 64


class _Pending:
    """Entries set since the last assembly.

    base    the CSR arrays at the first entry that had no slot (their values
            start the fold of their (row, col)), or None
    chunks  logged blocks in call order: (rows, cols, values, add) arrays
    single  (row, col) -> value folded as the reference's dict does; a key
            is here only while no logged block holds it (a single entry set
            after a block was logged folds everything first)
    """

    __slots__ = ("base", "chunks", "single")

    def __init__(self, base=None):
        self.base = base
        self.chunks = []
        self.single = {}

    def base_value(self, row, col):
        if self.base is None:
            return 0.0
        irow, icol, data = self.base
        lo, hi = int(irow[row]), int(irow[row + 1])
        pos = lo + int(np.searchsorted(icol[lo:hi], col))
        if pos < hi and int(icol[pos]) == col:
            return float(data[pos])
        return 0.0

    def flush_single(self):
        if self.single:
            keys = np.array(list(self.single.keys()), dtype=np.int64).reshape(-1, 2)
            vals = np.fromiter(self.single.values(), dtype=np.float64, count=len(self.single))
            self.chunks.append((keys[:, 0].copy(), keys[:, 1].copy(), vals,
                                np.zeros(len(vals), dtype=np.uint8)))
            self.single = {}

    def log(self, nrows):
        """All entries in fold order: the base CSR (inserts), the blocks, then
        the single entries (inserts of their folded values)."""
        self.flush_single()
        parts = []
        if self.base is not None:
            irow, icol, data = self.base
            rows = np.repeat(np.arange(nrows, dtype=np.int64), np.diff(irow))
            parts.append((rows, icol, data, np.zeros(len(data), dtype=np.uint8)))
        parts.extend(self.chunks)
        if not parts:
            e = np.zeros(0, dtype=np.int64)
            return e, e, np.zeros(0), np.zeros(0, dtype=np.uint8)
        return tuple(np.concatenate([p[k] for p in parts]) for k in range(4))


def _fold_host(nrows, ncols, rows, cols, vals, add):
    """CSR of an entry log on the host (same fold as gp_coo_assemble)."""
    key = rows * ncols + cols
    order = np.argsort(key, kind="stable")
    ks, vs, ad = key[order], vals[order], add[order]
    head = np.flatnonzero(np.r_[True, ks[1:] != ks[:-1]]) if len(ks) else np.zeros(0, np.int64)
    count = np.diff(np.r_[head, len(ks)])
    out = np.where(ad[head] != 0, 0.0 + vs[head], vs[head])
    for s in np.flatnonzero(count > 1):
        acc = 0.0
        for q in range(int(head[s]), int(head[s]) + int(count[s])):
            acc = acc + float(vs[q]) if ad[q] else float(vs[q])
        out[s] = acc
    ukey = ks[head]
    r, c = ukey // max(ncols, 1), ukey % max(ncols, 1)
    indptr = np.zeros(nrows + 1, dtype=np.int64)
    if nrows:
        indptr[1:] = np.cumsum(np.bincount(r, minlength=nrows))
    return indptr, c.astype(np.int64), out.astype(np.float64)


def _fold(nrows, ncols, rows, cols, vals, add):
    n = len(rows)
    if n >= DEVICE_ASSEMBLY_MIN and dev.has_device():
        indptr = np.zeros(nrows + 1, dtype=np.int64)
        indices = np.zeros(max(n, 1), dtype=np.int64)
        out = np.zeros(max(n, 1), dtype=np.float64)
        nnz = ctypes.c_int64()
        rows, cols = np.ascontiguousarray(rows, np.int64), np.ascontiguousarray(cols, np.int64)
        vals, add = np.ascontiguousarray(vals, np.float64), np.ascontiguousarray(add, np.uint8)
        check(lib().gp_coo_assemble(nrows, ncols, n, rows.ctypes.data, cols.ctypes.data,
                                    vals.ctypes.data, add.ctypes.data, indptr.ctypes.data,
                                    indices.ctypes.data, out.ctypes.data, ctypes.byref(nnz),
                                    dev.stream_ptr()))
        return indptr, indices[: nnz.value].copy(), out[: nnz.value].copy()
    return _fold_host(nrows, ncols, rows, cols, vals, add)


class MatType:
    AIJ = "aij"
    SEQAIJ = "seqaij"
    MPIAIJ = "mpiaij"
    SBAIJ = "sbaij"
    DENSE = "dense"
    SHELL = "shell"
    NEST = "nest"
    AIJCUSPARSE = "seqaijcusparse"


class MatInfoType:
    NNZ = "nz_allocated"
    NZ_USED = "nz_used"
    NNZ_USED = "nz_used"
    NNZ_ALLOCATED = "nz_allocated"
    FACTOR_NONZERO = "factor_nonz"
    ZERO_TOLERANCE = "rcond"
    ROW_ZERO_TOLERANCE = "rcond"


class MatStructures:
    SAME_NONZERO_PATTERN = 2
    DIFFERENT_NONZERO_PATTERN = 0
    SAME = SAME_NONZERO_PATTERN
    DIFFERENT = DIFFERENT_NONZERO_PATTERN


class MatOrderingType:
    NATURAL = "natural"
    ND = "nd"
    RCM = "rcm"
    MD = "md"
    ROWLENGTH = "rowlength"
    QMD = "qmd"
    AMD = "amd"
    METISND = "metisnd"
    EXTERNAL = "external"
    NATURAL_OR_ND = "natural_or_nd"


class MatSORType:
    ZERO_INITIAL_GUESS = 16
    FORWARD_SWEEP = 1
    BACKWARD_SWEEP = 2
    LOCAL_FORWARD_SWEEP = 4
    LOCAL_BACKWARD_SWEEP = 8
    LOCAL_SYMMETRIC_SWEEP = 12
    EISENSTAT = 32
    APPLY_UPPER = 64
    APPLY_LOWER = 128
    FORWARD = 1
    BACKWARD = 2
    SYMMETRIC = 3
    LOCAL_FORWARD = 4
    LOCAL_BACKWARD = 8
    LOCAL_SYMMETRIC = 12


class Mat:
    """A sequential AIJ matrix: host assembly, GPU algebra."""

    Type = MatType
    InfoType = MatInfoType
    OrderingType = MatOrderingType
    Structure = MatStructures
    SORType = MatSORType

    def __init__(self):
        self._irow = None
        self._icol = None
        self._data = None
        self._nrows = 0
        self._ncols = 0
        self._nnz_used = 0
        self._pending = None
        self._assembled = False
        # device mirror
        self._gp = None
        self._pver = 0       # pattern version of the host arrays
        self._vver = 0       # values version of the host arrays
        self._gp_pver = -1
        self._gp_vver = -1

    def __del__(self):
        self._drop_device()

    # ---------------------------------------------------------- device
    def _drop_device(self):
        h = getattr(self, "_gp", None)
        if h is not None:
            try:
                lib().gp_mat_destroy(h)
            except Exception:
                pass
        self._gp = None

    def _touch_values(self):
        self._vver += 1

    def _touch_pattern(self):
        self._pver += 1
        self._vver += 1

    def _device(self):
        """The gp_mat handle, current with the host arrays."""
        self._materialize()
        if self._gp is not None and self._gp_pver == self._pver:
            if self._gp_vver != self._vver:
                nnz = self._nnz_used
                vals = np.ascontiguousarray(self._data[:nnz], dtype=np.float64)
                check(lib().gp_mat_set_values(self._gp, vals.ctypes.data if nnz else None, 0,
                                              dev.stream_ptr()))
                dev.synchronize()
                self._gp_vver = self._vver
            return self._gp
        self._drop_device()
        dev.require_device()
        n, nnz = self._nrows, self._nnz_used
        irow = np.ascontiguousarray(self._irow[: n + 1], dtype=np.int64)
        icol = np.ascontiguousarray(self._icol[:nnz], dtype=np.int64)
        vals = np.ascontiguousarray(self._data[:nnz], dtype=np.float64)
        h = ctypes.c_void_p()
        check(lib().gp_mat_create(ctypes.byref(h), n, self._ncols, nnz, irow.ctypes.data,
                                  icol.ctypes.data if nnz else None,
                                  vals.ctypes.data if nnz else None))
        self._gp = h.value
        self._gp_pver, self._gp_vver = self._pver, self._vver
        return self._gp

    def _values_tensor(self):
        """Device address of the values array (shares memory)."""
        p = ctypes.c_void_p()
        check(lib().gp_mat_values_ptr(self._device(), ctypes.byref(p)))
        return p.value

    # ---------------------------------------------------------- creation
    def create(self, comm=None) -> "Mat":
        return self

    def createSeqAIJ(self, size, bsize=None, nnz=None, comm=None) -> "Mat":
        """Create an empty sequential AIJ matrix; `size` is the number of rows
        or a (rows, cols) pair."""
        if isinstance(size, (tuple, list)):
            m, n = int(size[0]), int(size[1])
        else:
            m = n = int(size)
        per_row = 1 if nnz is None else int(nnz)
        self._nrows, self._ncols = m, n
        self._irow = np.zeros(m + 1, dtype=np.int64)
        self._icol = np.zeros(max(m * per_row, 1), dtype=np.int64)
        self._data = np.zeros(max(m * per_row, 1), dtype=np.float64)
        self._nnz_used = 0
        self._assembled = True
        self._pending = _Pending()
        self._touch_pattern()
        return self

    def createAIJ(self, size, bsize=None, nnz=None, comm=None) -> "Mat":
        return self.createSeqAIJ(size, bsize, nnz, comm)

    def setSizes(self, size, bsize=None) -> "Mat":
        if isinstance(size, (tuple, list)):
            r, c = size[0], size[1]
            self._nrows = int(r[0] if isinstance(r, (tuple, list)) else r)
            self._ncols = int(c[0] if isinstance(c, (tuple, list)) else c)
        else:
            self._nrows = self._ncols = int(size)
        if self._irow is None:
            self.createSeqAIJ((self._nrows, self._ncols))
        return self

    def setType(self, mat_type) -> "Mat":
        return self

    def setUp(self) -> "Mat":
        self._check()._materialize()
        self._assembled = True
        return self

    def setPreallocationNNZ(self, nnz) -> "Mat":
        return self

    def setOption(self, option, flag) -> None:
        return None

    def assemblyBegin(self, assembly=None) -> None:
        return None

    def assemblyEnd(self, assembly=None) -> None:
        self._materialize()
        self._assembled = True

    def assemble(self, assembly=None) -> "Mat":
        self.assemblyEnd()
        return self

    def destroy(self) -> "Mat":
        self._drop_device()
        self._irow = None
        return self

    def _check(self):
        if self._irow is None:
            raise RuntimeError("Mat has not been created")
        return self

    def duplicate(self, copy: bool = False) -> "Mat":
        self._materialize()
        out = Mat()
        out._nrows, out._ncols = self._nrows, self._ncols
        out._irow = self._irow.copy()
        out._icol = self._icol.copy()
        out._data = self._data.copy() if copy else np.zeros_like(self._data)
        out._nnz_used = self._nnz_used
        out._assembled = self._assembled
        out._touch_pattern()
        return out

    def copy(self, result=None, structure=None) -> "Mat":
        """Copy into `result` (a duplicate when None).  With
        DIFFERENT_NONZERO_PATTERN the target keeps its own pattern and takes
        the source's value at each of its slots (zero where the source has
        none), as the reference's copy does."""
        self._materialize()
        target = self.duplicate() if result is None else result
        if structure == MatStructures.DIFFERENT_NONZERO_PATTERN:
            target._materialize()
            if target.getSize() != self.getSize():
                raise ValueError(f"incompatible sizes: {self.getSize()} into {target.getSize()}")
            src = {}
            for i in range(self._nrows):
                for j in range(int(self._irow[i]), int(self._irow[i + 1])):
                    src[(i, int(self._icol[j]))] = float(self._data[j])
            for i in range(target._nrows):
                for j in range(int(target._irow[i]), int(target._irow[i + 1])):
                    target._data[j] = src.get((i, int(target._icol[j])), 0.0)
            target._touch_values()
            return target
        target._nrows, target._ncols = self._nrows, self._ncols
        target._irow = self._irow.copy()
        target._icol = self._icol.copy()
        target._data = self._data.copy()
        target._nnz_used = self._nnz_used
        target._assembled = self._assembled
        target._pending = None
        target._touch_pattern()
        return target

    # ---------------------------------------------------------- accessors
    def getType(self) -> str:
        return "seqaij"

    def getSize(self):
        return (self._nrows, self._ncols)

    def getLocalSize(self):
        return (self._nrows, self._ncols)

    def getSizes(self):
        return ((self._nrows, self._nrows), (self._ncols, self._ncols))

    def getOwnershipRange(self):
        return (0, self._nrows)

    def getOwnershipRangeColumn(self):
        return (0, self._ncols)

    def getBlockSize(self) -> int:
        return 1

    def getNNZ(self) -> int:
        self._materialize()
        return int(self._nnz_used)

    def getInfo(self, info=None) -> dict:
        self._materialize()
        return {"nz_allocated": int(len(self._data)), "nz_used": int(self._nnz_used),
                "rcond": 0.0}

    @property
    def irow(self) -> np.ndarray:
        self._materialize()
        return self._irow

    @property
    def icol(self) -> np.ndarray:
        self._materialize()
        return self._icol

    @property
    def data(self) -> np.ndarray:
        self._materialize()
        return self._data

    def getValuesCSR(self):
        self._materialize()
        nnz = int(self._nnz_used)
        return (self._irow[: self._nrows + 1].copy(), self._icol[:nnz].copy(),
                self._data[:nnz].copy())

    def setValuesCSR(self, indptr, indices, data=None) -> "Mat":
        """Install CSR arrays (row starts, column indices, values)."""
        irow = np.asarray(indptr, dtype=np.int64)
        icol = np.asarray(indices, dtype=np.int64)
        vals = (np.zeros(0, dtype=np.float64) if data is None
                else np.asarray(data, dtype=np.float64))
        if self._irow is None:
            self.createSeqAIJ((len(irow) - 1, self._ncols or len(irow) - 1))
        if len(irow) != self._nrows + 1:
            raise ValueError(
                f"incompatible array sizes: indptr has {len(irow)} entries,"
                f" {self._nrows + 1} are needed"
            )
        if len(icol) != len(vals):
            raise ValueError(
                f"incompatible array sizes: {len(icol)} indices but {len(vals)} values"
            )
        nnz = int(irow[-1])
        if self._data.size < nnz:
            self._data = np.zeros(nnz, dtype=np.float64)
            self._icol = np.zeros(nnz, dtype=np.int64)
        self._irow[:] = irow
        self._icol[:nnz] = icol[:nnz]
        self._data[:nnz] = vals[:nnz]
        self._nnz_used = nnz
        self._pending = None
        self._touch_pattern()
        return self

    def _materialize(self):
        """Fold the pending entries into CSR (Mat.py:383-413 of the
        reference: sorted by (row, col), each entry's ops in call order)."""
        if self._pending is None:
            return
        rows, cols, vals, add = self._pending.log(self._nrows)
        irow, icol, data = _fold(self._nrows, self._ncols, rows, cols, vals, add)
        total = int(irow[-1])
        if total == 0:
            icol, data = np.zeros(1, dtype=np.int64), np.zeros(1, dtype=np.float64)
        self._irow, self._icol, self._data = irow, icol, data
        self._nnz_used = total
        self._pending = None
        self._touch_pattern()

    def _locate(self, row: int, col: int) -> int:
        if row < 0 or row >= self._nrows or col < 0 or col >= self._ncols:
            return -1
        lo, hi = int(self._irow[row]), int(self._irow[row + 1])
        pos = lo + int(np.searchsorted(self._icol[lo:hi], col))
        if pos >= hi or int(self._icol[pos]) != col:
            return -1
        return pos

    def _entry(self, row: int, col: int) -> float:
        p = self._pending
        if p is not None:
            v = p.single.get((row, col))
            if v is not None:
                return float(v)
            if not p.chunks:
                return p.base_value(row, col)
            self._materialize()
        j = self._locate(row, col)
        return 0.0 if j < 0 else float(self._data[j])

    def getValue(self, row, col) -> float:
        return self._entry(int(row), int(col))

    def getValues(self, rows, cols, values=None) -> np.ndarray:
        out = np.array([[self.getValue(r, c) for c in cols] for r in rows], dtype=np.float64)
        if values is not None:
            values[:] = out
            return values
        return out

    def _spill(self):
        """Keep the CSR entries as the base of the pending entries, so later
        entries fold onto them."""
        if self._pending is not None:
            return
        nnz = self._nnz_used
        self._pending = _Pending((self._irow[: self._nrows + 1].copy(),
                                  self._icol[:nnz].copy(), self._data[:nnz].copy()))

    def _setValue(self, row, col, value, addv):
        if row < 0 or row >= self._nrows or col < 0 or col >= self._ncols:
            raise ValueError(f"entry ({row}, {col}) is out of range")
        if self._pending is None:
            j = self._locate(row, col)
            if j >= 0:  # existing slot: values only
                self._data[j] = self._data[j] + value if addv else value
                self._touch_values()
                return
        self._spill()
        p = self._pending
        cur = p.single.get((row, col))
        if cur is None:
            if p.chunks:  # the entry may sit in a logged block: fold first
                self._materialize()
                return self._setValue(row, col, value, addv)
            cur = p.base_value(row, col)
        p.single[(row, col)] = cur + value if addv else value

    def setValue(self, row, col, value, addv=None) -> None:
        self._setValue(int(row), int(col), float(value), addv is not None)

    def setValues(self, rows, cols, values, addv=None, insertmode=None) -> None:
        rows, cols, vals = list(rows), list(cols), np.ravel(np.asarray(values, dtype=np.float64))
        need = len(rows) * len(cols)
        if len(vals) < need:
            raise ValueError(
                f"incompatible array sizes: ni={len(rows)}, nj={len(cols)}, nv={len(vals)};"
                f" at least {need} values are needed"
            )
        add = addv is not None
        if need < BLOCK_LOG_MIN:
            for i, r in enumerate(rows):
                for j, c in enumerate(cols):
                    self._setValue(int(r), int(c), float(vals[i * len(cols) + j]), add)
            return
        r = np.asarray(rows, dtype=np.int64).ravel()
        c = np.asarray(cols, dtype=np.int64).ravel()
        R, C = np.repeat(r, len(c)), np.tile(c, len(r))
        bad = (R < 0) | (R >= self._nrows) | (C < 0) | (C >= self._ncols)
        if bad.any():
            k = int(np.argmax(bad))
            raise ValueError(f"entry ({int(R[k])}, {int(C[k])}) is out of range")
        self._log_block(R, C, np.array(vals[:need], dtype=np.float64), add)

    def _log_block(self, R, C, V, add):
        """A block of entries in call order (rows R, columns C, values V)."""
        if self._pending is None:
            # every entry has a slot and no slot repeats: values in place
            pos = self._locate_many(R, C)
            if (pos >= 0).all() and len(np.unique(pos)) == len(pos):
                if add:
                    self._data[pos] = self._data[pos] + V
                else:
                    self._data[pos] = V
                self._touch_values()
                return
        self._spill()
        p = self._pending
        p.flush_single()
        p.chunks.append((R, C, V, np.full(len(R), 1 if add else 0, dtype=np.uint8)))

    def _locate_many(self, R, C):
        """Slots of the entries (R, C) in the CSR arrays (-1 where absent)."""
        nnz = self._nnz_used
        key = self._icol[:nnz] + np.repeat(np.arange(self._nrows, dtype=np.int64),
                                           np.diff(self._irow[: self._nrows + 1])) * self._ncols
        want = R * self._ncols + C
        pos = np.searchsorted(key, want)
        ok = pos < nnz
        ok[ok] = key[pos[ok]] == want[ok]
        return np.where(ok, pos, -1)

    def setValueBlocked(self, rows, cols, value, addv=None) -> None:
        add = addv is not None
        for r in list(rows):
            for c in list(cols):
                self._setValue(int(r), int(c), float(value), add)

    def setValuesBlocked(self, rows, cols, values, addv=None) -> None:
        self.setValues(rows, cols, values, addv)

    def zeroEntries(self) -> None:
        self._check()._materialize()
        self._data[:] = 0.0
        self._touch_values()

    def _dense(self) -> np.ndarray:
        self._materialize()
        out = np.zeros((self._nrows, self._ncols), dtype=np.float64)
        for i in range(self._nrows):
            for j in range(int(self._irow[i]), int(self._irow[i + 1])):
                out[i, int(self._icol[j])] += float(self._data[j])
        return out

    # ---------------------------------------------------------- algebra (GPU)
    def _check_len(self, v: Vec, n: int, what: str) -> Vec:
        if v._size() != n:
            raise ValueError(f"incompatible sizes: {what} has {v._size()} entries, {n} needed")
        return v

    def mult(self, x: Vec, y: Vec = None) -> Vec:
        """y = A x."""
        self._materialize()
        self._check_len(x, self._ncols, "x")
        out = Vec().createSeq(self._nrows) if y is None else self._check_len(y, self._nrows, "y")
        if out is x:
            raise ValueError("output y may not alias the input x in mult")
        if self._nrows:
            h = self._device()
            check(lib().gp_mat_mult(h, x._dptr(), out._optr(), dev.stream_ptr()))
        return out

    def multAdd(self, x: Vec, v: Vec, y: Vec = None) -> Vec:
        """y = A x + v."""
        self._materialize()
        self._check_len(x, self._ncols, "x")
        self._check_len(v, self._nrows, "v")
        out = Vec().createSeq(self._nrows) if y is None else self._check_len(y, self._nrows, "y")
        if out is x:
            raise ValueError("output y may not alias the input x in multAdd")
        if self._nrows:
            h = self._device()
            vp = v._dptr()
            check(lib().gp_mat_mult_add(h, x._dptr(), vp, out._wptr() if out is v else out._optr(),
                                        dev.stream_ptr()))
        return out

    def multTranspose(self, x: Vec, y: Vec = None) -> Vec:
        """y = A^T x."""
        self._materialize()
        self._check_len(x, self._nrows, "x")
        out = Vec().createSeq(self._ncols) if y is None else self._check_len(y, self._ncols, "y")
        if out is x:
            raise ValueError("output y may not alias the input x in multTranspose")
        if self._ncols:
            h = self._device()
            check(lib().gp_mat_mult_transpose(h, x._dptr() if self._nrows else 0,
                                              out._optr(), dev.stream_ptr()))
        return out

    def multTransposeAdd(self, x: Vec, v: Vec, y: Vec = None) -> Vec:
        """y = A^T x + v."""
        self._materialize()
        self._check_len(x, self._nrows, "x")
        self._check_len(v, self._ncols, "v")
        out = Vec().createSeq(self._ncols) if y is None else self._check_len(y, self._ncols, "y")
        if out is x:
            raise ValueError("output y may not alias the input x in multTransposeAdd")
        keep = v.copy() if out is v else v
        self.multTranspose(x, out)
        out.axpy(1.0, keep)
        return out

    def createVecLeft(self) -> Vec:
        return Vec().createSeq(self._nrows)

    def createVecRight(self) -> Vec:
        return Vec().createSeq(self._ncols)

    def getVecs(self):
        return (self.createVecRight(), self.createVecLeft())

    def __call__(self, x, y=None):
        return self.mult(x, y)

    def getDiagonal(self, result: Vec = None) -> Vec:
        self._materialize()
        out = Vec().createSeq(self._nrows) if result is None else \
            self._check_len(result, self._nrows, "result")
        if self._nrows:
            check(lib().gp_mat_get_diagonal(self._device(), out._optr(), dev.stream_ptr()))
        return out

    def createDiagonal(self, d: Vec) -> "Mat":
        arr = d.getArray(readonly=True)
        n = len(arr)
        out = Mat().createSeqAIJ(n, nnz=1)
        out.setValuesCSR(np.arange(n + 1), np.arange(n), arr.copy())
        return out

    def createTranspose(self, mat=None) -> "Mat":
        return _transpose(self if mat is None else mat)

    def transpose(self, out: "Mat" = None) -> "Mat":
        return _transpose(self)

    def scale(self, alpha) -> None:
        self._check()._materialize()
        self._data[:] = self._data * float(alpha)
        self._touch_values()

    def equal(self, mat, tol: float = 0.0) -> bool:
        self._materialize()
        mat._materialize()
        if self.getSize() != mat.getSize():
            return False
        a, b = self.getValuesCSR(), mat.getValuesCSR()
        if not (np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])):
            return False
        return bool(np.allclose(a[2], b[2], rtol=0, atol=tol))

    def isSymmetric(self, tol: float = 0.0) -> bool:
        if self._nrows != self._ncols:
            return False
        return bool(np.allclose(self._dense(), self._dense().T, rtol=0, atol=tol))

    def isTranspose(self, mat=None, tol: float = 0.0) -> bool:
        other = self if mat is None else mat
        if self.getSize() != other.getSize()[::-1]:
            return False
        return bool(np.allclose(self._dense(), other._dense().T, rtol=0, atol=tol))

    def __matmul__(self, x):
        return self.mult(x)

    def __mul__(self, other):
        if not isinstance(other, Mat):
            return NotImplemented
        if self._ncols != other._nrows:
            raise ValueError(f"incompatible sizes: {self.getSize()} times {other.getSize()}")
        return from_dense(self._dense() @ other._dense())

    def __neg__(self):
        out = self.duplicate(copy=True)
        out.scale(-1.0)
        return out


def _transpose(m: Mat) -> Mat:
    """A^T in CSR (a stable sort by column, so each row of A^T lists its
    entries in ascending original row; Mat.py:682-716 of the reference).
    Large matrices are transposed on the GPU (gp_mat_transpose: the pattern
    by a stable radix sort, the values gathered through it)."""
    rows, cols, vals = m.getValuesCSR()
    nnz = len(cols)
    if nnz >= DEVICE_ASSEMBLY_MIN and dev.has_device():
        t = ctypes.c_void_p()
        check(lib().gp_mat_transpose(m._device(), ctypes.byref(t), dev.stream_ptr()))
        try:
            indptr = np.zeros(m._ncols + 1, dtype=np.int64)
            indices = np.zeros(nnz, dtype=np.int64)
            values = np.zeros(nnz, dtype=np.float64)
            check(lib().gp_mat_get_csr(t.value, indptr.ctypes.data, indices.ctypes.data,
                                       values.ctypes.data, dev.stream_ptr()))
        finally:
            lib().gp_mat_destroy(t.value)
        out = Mat().createSeqAIJ((m._ncols, m._nrows), nnz=1)
        out.setValuesCSR(indptr, indices, values)
        return out
    row_of = np.repeat(np.arange(m._nrows, dtype=np.int64), np.diff(rows))
    order = np.argsort(cols, kind="stable")
    counts = np.bincount(cols, minlength=m._ncols) if nnz else np.zeros(m._ncols, np.int64)
    indptr = np.zeros(m._ncols + 1, dtype=np.int64)
    indptr[1:] = np.cumsum(counts)
    out = Mat().createSeqAIJ((m._ncols, m._nrows), nnz=1)
    out.setValuesCSR(indptr, row_of[order], vals[order])
    return out


def from_dense(array, mat=None) -> Mat:
    """CSR from a dense 2-D array (nonzero entries, row-major order)."""
    arr = np.ascontiguousarray(array, dtype=np.float64)
    if arr.ndim != 2:
        raise ValueError("expected a 2-D array")
    n, m = arr.shape
    out = mat if mat is not None else Mat()
    out.createSeqAIJ((n, m))
    if arr.size >= DEVICE_ASSEMBLY_MIN and dev.has_device():
        cap = int(np.count_nonzero(arr))
        indptr = np.zeros(n + 1, dtype=np.int64)
        indices = np.zeros(max(cap, 1), dtype=np.int64)
        values = np.zeros(max(cap, 1), dtype=np.float64)
        nnz = ctypes.c_int64()
        check(lib().gp_dense_to_csr(n, m, arr.ctypes.data, cap, indptr.ctypes.data,
                                    indices.ctypes.data, values.ctypes.data, ctypes.byref(nnz),
                                    dev.stream_ptr()))
        out.setValuesCSR(indptr, indices[: nnz.value], values[: nnz.value])
        return out
    rr, cc = np.nonzero(arr)
    indptr = np.zeros(n + 1, dtype=np.int64)
    indptr[1:] = np.cumsum(np.bincount(rr, minlength=n)) if n else []
    out.setValuesCSR(indptr, cc.astype(np.int64), arr[rr, cc])
    return out
