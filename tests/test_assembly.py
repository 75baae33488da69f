"""Matrix assembly: pending entries, blocks, the device fold, transpose and
from_dense.

The reference keeps entries set after an assembly in a dict of rows,
folding each (row, col) in call order -- INSERT sets, ADD adds to the
current value, starting from 0.0 or the assembled value
(python/mojopetsc4py/PETSc/Mat.py:383-413, 434-439).  `DictModel` below
restates that rule; every sequence of setValue / setValues / getValue /
assemble calls must give the same CSR bit for bit, whether the entries go
one by one, as logged blocks folded on the host, or (GPU) folded by
gp_coo_assemble.
"""
import importlib

import numpy as np
import pytest

from mojopetsc4py import PETSc

M = importlib.import_module("mojopetsc4py.PETSc.Mat")  # the module (PETSc.Mat is the class)


class DictModel:
    """The reference's pending-entry rule, entry by entry."""

    def __init__(self, n, m):
        self.n, self.m = n, m
        self.d = {}

    def set(self, r, c, v, add):
        cur = self.d.get((r, c), 0.0)
        self.d[(r, c)] = cur + v if add else v

    def get(self, r, c):
        return self.d.get((r, c), 0.0)

    def csr(self):
        keys = sorted(self.d)
        indptr = np.zeros(self.n + 1, dtype=np.int64)
        for r, _ in keys:
            indptr[r + 1] += 1
        indptr = np.cumsum(indptr)
        cols = np.array([c for _, c in keys], dtype=np.int64)
        vals = np.array([self.d[k] for k in keys], dtype=np.float64)
        return indptr, cols, vals


def _check(A, model):
    ip, ix, v = A.getValuesCSR()
    wip, wix, wv = model.csr()
    np.testing.assert_array_equal(ip, wip)
    np.testing.assert_array_equal(ix, wix)
    np.testing.assert_array_equal(v.view(np.int64), wv.view(np.int64))  # bits, -0.0 too


def _script(rng, n, m, steps, block):
    """A random call sequence: single entries, blocks, reads, assemblies."""
    out = []
    for _ in range(steps):
        kind = rng.choice(["single", "block", "get", "assemble"], p=[0.45, 0.35, 0.15, 0.05])
        add = bool(rng.integers(2))
        if kind == "single":
            out.append(("single", int(rng.integers(n)), int(rng.integers(m)),
                        float(rng.choice([rng.normal(), -0.0, 0.0, 1e-300])), add))
        elif kind == "block":
            rows = rng.integers(0, n, rng.integers(1, block))
            cols = rng.integers(0, m, rng.integers(1, block))
            vals = rng.normal(size=len(rows) * len(cols))
            vals[rng.random(len(vals)) < 0.05] = -0.0
            out.append(("block", rows, cols, vals, add))
        elif kind == "get":
            out.append(("get", int(rng.integers(n)), int(rng.integers(m))))
        else:
            out.append(("assemble",))
    return out


def _run(script, n, m):
    A = PETSc.Mat().createAIJ((n, m))
    model = DictModel(n, m)
    for op in script:
        if op[0] == "single":
            _, r, c, v, add = op
            A.setValue(r, c, v, addv=True if add else None)
            model.set(r, c, v, add)
        elif op[0] == "block":
            _, rows, cols, vals, add = op
            A.setValues(rows, cols, vals, addv=True if add else None)
            for i, r in enumerate(rows):
                for j, c in enumerate(cols):
                    model.set(int(r), int(c), float(vals[i * len(cols) + j]), add)
        elif op[0] == "get":
            _, r, c = op
            assert np.float64(A.getValue(r, c)).view(np.int64) == \
                np.float64(model.get(r, c)).view(np.int64)
        else:
            A.assemble()
    A.assemble()
    return A, model


@pytest.mark.parametrize("seed", range(6))
def test_pending_entries_follow_the_reference_rule(seed, monkeypatch):
    # host folds only, whatever the device
    monkeypatch.setattr(M, "DEVICE_ASSEMBLY_MIN", 1 << 62)
    rng = np.random.default_rng(seed)
    n, m = int(rng.integers(5, 40)), int(rng.integers(5, 40))
    A, model = _run(_script(rng, n, m, 120, 12), n, m)
    _check(A, model)


def test_blocks_into_an_assembled_pattern_update_in_place(monkeypatch):
    monkeypatch.setattr(M, "DEVICE_ASSEMBLY_MIN", 1 << 62)
    n = 30
    A = PETSc.Mat().createAIJ((n, n))
    rows = np.arange(n)
    A.setValues(rows, rows, np.zeros(n * n))  # dense pattern, values 0
    A.assemble()
    model = DictModel(n, n)
    for r in range(n):
        for c in range(n):
            model.set(r, c, 0.0, False)
    rng = np.random.default_rng(1)
    for _ in range(5):
        rr = rng.permutation(n)[:10]
        cc = rng.permutation(n)[:9]
        vals = rng.normal(size=90)
        A.setValues(rr, cc, vals, addv=True)
        for i, r in enumerate(rr):
            for j, c in enumerate(cc):
                model.set(int(r), int(c), float(vals[i * 9 + j]), True)
    A.assemble()
    _check(A, model)


def test_out_of_range_block_entry_raises():
    A = PETSc.Mat().createAIJ((10, 10))
    with pytest.raises(ValueError, match=r"entry \(10, 0\) is out of range"):
        A.setValues(np.arange(11), np.arange(8), np.ones(88))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(3))
def test_device_fold_matches_the_host_fold(seed):
    """Logs long enough for gp_coo_assemble: same CSR bits as the host fold
    and the reference rule."""
    rng = np.random.default_rng(100 + seed)
    n, m = 3000, 2500
    script = _script(rng, n, m, 60, 120)
    A, model = _run(script, n, m)
    _check(A, model)
    # and the raw fold of one large log, device against host
    k = 200_000
    rows = rng.integers(0, n, k)
    cols = rng.integers(0, 40, k) * 50 + rng.integers(0, 3, k)  # many repeats
    vals = rng.normal(size=k)
    vals[rng.random(k) < 0.01] = -0.0
    add = (rng.random(k) < 0.7).astype(np.uint8)
    d = M._fold(n, m, rows, cols, vals, add)
    h = M._fold_host(n, m, rows, cols, vals, add)
    for a, b in zip(d, h):
        np.testing.assert_array_equal(np.asarray(a).view(np.int64), np.asarray(b).view(np.int64))


@pytest.mark.gpu
def test_device_fold_rejects_out_of_range_entries():
    from mojopetsc4py._lib import GPError

    rows = np.array([0] * 40000 + [7], dtype=np.int64)
    cols = np.zeros(len(rows), dtype=np.int64)
    with pytest.raises(GPError, match="out of range"):
        M._fold(5, 5, rows, cols, np.ones(len(rows)), np.zeros(len(rows), dtype=np.uint8))


@pytest.mark.gpu
def test_device_transpose_and_from_dense():
    rng = np.random.default_rng(7)
    n, m = 700, 900
    dense = rng.normal(size=(n, m))
    dense[rng.random((n, m)) < 0.9] = 0.0
    dense[0, :] = 0.0  # an empty row
    A = M.from_dense(dense)  # n * m entries: the device path
    ip, ix, v = A.getValuesCSR()
    rr, cc = np.nonzero(dense)
    np.testing.assert_array_equal(ix, cc)
    np.testing.assert_array_equal(v, dense[rr, cc])
    np.testing.assert_array_equal(np.diff(ip), np.count_nonzero(dense, axis=1))
    T = A.transpose()  # nnz >= the device threshold
    assert len(ix) >= M.DEVICE_ASSEMBLY_MIN
    tip, tix, tv = T.getValuesCSR()
    np.testing.assert_array_equal(T._dense(), dense.T)
    rr, cc = np.nonzero(dense.T)
    np.testing.assert_array_equal(tix, cc)
    np.testing.assert_array_equal(tv, dense.T[rr, cc])
