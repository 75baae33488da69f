"""GPU kernels against the CPU oracle on identical inputs.

SpMV, SpMV-add, SpMV-transpose, the diagonal, the elementwise Vec maps, the
preconditioner applies and the incomplete factorisations are the same
rounded operations in the same order as the sequential loops, so they are
compared bit for bit.  Reductions sum in a different (fixed, parallel) order
and are compared to 1e-13 relative."""
import numpy as np
import pytest

import oracle as O
from helpers import dense_to_csr, nonsym_banded, spd_dense, tridiag_dense
from mojopetsc4py import PETSc, gallery

pytestmark = pytest.mark.gpu


def a(x):
    return x.ctypes.data


def mat(ip, ix, v, ncols=None):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, ncols or n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    return A


def vec(x):
    return PETSc.Vec().createWithArray(np.asarray(x, dtype=np.float64))


MATRICES = {
    "poisson3d_24": lambda: gallery.laplacian_3d(24),
    "convdiff_12": lambda: gallery.convection_diffusion_3d(12),
    "nonsym_200": lambda: dense_to_csr(nonsym_banded(200, 4)),
}


@pytest.mark.parametrize("name", list(MATRICES))
def test_spmv_bit_exact(name):
    ip, ix, v = MATRICES[name]()
    ip64, ix64 = O.i64(ip), O.i64(ix)
    n = len(ip) - 1
    x = np.random.default_rng(1).normal(size=n)
    A = mat(ip, ix, v)
    y = A.mult(vec(x)).getArray()
    want = np.zeros(n)
    O.lib().mp_mat_mult(a(x), a(want), a(ip64), a(ix64), a(v), n)
    np.testing.assert_array_equal(y, want)
    # multAdd starts each row from v
    w = np.random.default_rng(2).normal(size=n)
    y2 = A.multAdd(vec(x), vec(w)).getArray()
    want2 = w.copy()
    O.lib().mp_mat_mult_add(a(x), a(want2), a(ip64), a(ix64), a(v), n)
    np.testing.assert_array_equal(y2, want2)
    # transpose: the gather over A^T adds in the scatter's order
    yt = A.multTranspose(vec(x)).getArray()
    want3 = np.zeros(n)
    O.lib().mp_mat_mult_transpose(a(x), a(want3), a(ip64), a(ix64), a(v), n, n)
    np.testing.assert_array_equal(yt, want3)
    d = A.getDiagonal().getArray()
    want4 = np.zeros(n)
    O.lib().mp_mat_get_diagonal(a(want4), a(ip64), a(ix64), a(v), n)
    np.testing.assert_array_equal(d, want4)


def _index_bytes(A):
    import ctypes

    from mojopetsc4py._lib import check, lib

    b = ctypes.c_int32()
    check(lib().gp_mat_spmv_index_bytes(A._device(), ctypes.byref(b)))
    return b.value


@pytest.mark.parametrize("far", [False, True])
def test_spmv_column_offsets_of_16_bits_and_wide_bands(far):
    """Row-form matrices whose every |column - row| fits 16 bits are read
    through row-relative 16-bit offsets; one entry 40000 columns away keeps
    32-bit columns.  Both give the oracle's products bit for bit, in the
    standalone multiply and inside a fused CG solve."""
    ip, ix, v = gallery.laplacian_3d(36)  # n = 46656: offsets up to 1296
    n = len(ip) - 1
    if far:
        # add a symmetric pair (0, 40000) / (40000, 0) with a small value
        rows = [list(ix[ip[i]:ip[i + 1]]) for i in range(n)]
        vals = [list(v[ip[i]:ip[i + 1]]) for i in range(n)]
        for r, c in ((0, 40000), (40000, 0)):
            k = int(np.searchsorted(rows[r], c))
            rows[r].insert(k, c)
            vals[r].insert(k, -1e-3)
        ip = np.zeros(n + 1, np.int32)
        ip[1:] = np.cumsum([len(r) for r in rows])
        ix = np.concatenate(rows).astype(np.int32)
        v = np.concatenate(vals)
    A = mat(ip, ix, v)
    assert _index_bytes(A) == (4 if far else 2)
    x = np.random.default_rng(4).normal(size=n)
    y = A.mult(vec(x)).getArray()
    want = np.zeros(n)
    ip64, ix64 = O.i64(ip), O.i64(ix)  # kept alive across the call
    O.lib().mp_mat_mult(a(x), a(want), a(ip64), a(ix64), a(v), n)
    np.testing.assert_array_equal(y, want)
    b = np.random.default_rng(5).uniform(-1, 1, n)
    ksp = PETSc.KSP().create()
    ksp.setType("cg")
    ksp.getPC().setType("jacobi")
    ksp.setOperators(A)
    ksp.setTolerances(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=2000)
    xv = PETSc.Vec().createSeq(n)
    ksp.solve(vec(b), xv)
    ref = O.solve("cg", ip, ix, v, b, pc_type="jacobi", rtol=1e-10, atol=1e-50, divtol=1e30,
                  max_it=2000)
    assert ksp.getIterationNumber() == ref["its"]
    np.testing.assert_array_equal(xv.getArray(), ref["x"])


@pytest.mark.fma
def test_fused_cg_reads_16_bit_column_offsets():
    """The fused CG's SpMV (the timed path) on a matrix with 16-bit column
    offsets: the oracle's iteration count and reason, iterate within 1e-10."""
    ip, ix, v = gallery.laplacian_3d(36)
    n = len(ip) - 1
    A = mat(ip, ix, v)
    assert _index_bytes(A) == 2
    b = np.random.default_rng(6).uniform(-1, 1, n)
    ksp = PETSc.KSP().create()
    ksp.setType("cg")
    ksp.getPC().setType("jacobi")
    ksp.setOperators(A)
    ksp.setTolerances(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=2000)
    xv = PETSc.Vec().createSeq(n)
    ksp.solve(vec(b), xv)
    ref = O.solve("cg", ip, ix, v, b, pc_type="jacobi", rtol=1e-10, atol=1e-50, divtol=1e30,
                  max_it=2000)
    assert (ksp.getIterationNumber(), ksp.getConvergedReason()) == (ref["its"], ref["reason"])
    rel = np.linalg.norm(xv.getArray() - ref["x"]) / np.linalg.norm(ref["x"])
    assert rel <= 1e-10, rel


@pytest.mark.fma
def test_long_rows_are_summed_by_segments_in_the_fused_arithmetic():
    """Rows longer than 2048 slots in the row-stream form are summed by
    segments (one CTA a segment, a fixed tree, the segments in order): within
    rounding of the reference's products, the same bits run to run, and a CG
    solve with the oracle's iteration count and an iterate within 1e-10."""
    ip, ix, v = gallery.hub_laplacian(20000, 4, 5000)
    n = len(ip) - 1
    assert np.diff(ip).max() > 2048
    ip64, ix64 = O.i64(ip), O.i64(ix)
    A = mat(ip, ix, v)
    x = np.random.default_rng(4).normal(size=n)
    y = A.mult(vec(x)).getArray()
    want = np.zeros(n)
    O.lib().mp_mat_mult(a(x), a(want), a(ip64), a(ix64), a(v), n)
    scale = np.zeros(n)
    np.add.at(scale, np.repeat(np.arange(n), np.diff(ip)), np.abs(v * x[ix]))
    assert np.all(np.abs(y - want) <= 1e-14 * scale + 1e-300)
    np.testing.assert_array_equal(A.mult(vec(x)).getArray(), y)
    # A^T's long rows (A's dense columns) are split the same way: for this
    # symmetric matrix they hold A's rows in the same order, the same bits
    np.testing.assert_array_equal(A.multTranspose(vec(x)).getArray(), y)
    w = np.random.default_rng(5).normal(size=n)
    y2 = A.multAdd(vec(x), vec(w)).getArray()
    assert np.all(np.abs(y2 - (want + w)) <= 1e-14 * (scale + np.abs(w)) + 1e-300)
    b = np.random.default_rng(6).uniform(-1, 1, n)
    ksp = PETSc.KSP().create()
    ksp.setType("cg")
    ksp.getPC().setType("jacobi")
    ksp.setOperators(A)
    ksp.setTolerances(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=5000)
    xv = PETSc.Vec().createSeq(n)
    ksp.solve(vec(b), xv)
    ref = O.solve("cg", ip, ix, v, b, pc_type="jacobi", rtol=1e-10, atol=1e-50, divtol=1e30,
                  max_it=5000)
    assert (ksp.getIterationNumber(), ksp.getConvergedReason()) == (ref["its"], ref["reason"])
    rel = np.linalg.norm(xv.getArray() - ref["x"]) / np.linalg.norm(ref["x"])
    assert rel <= 1e-10, rel


def test_long_rows_keep_the_reference_fold_in_the_ordered_arithmetic():
    """The same matrix in the ordered arithmetic: every row, the long ones
    included, is folded slot by slot as the reference does (bit-identical)."""
    ip, ix, v = gallery.hub_laplacian(20000, 4, 5000)
    n = len(ip) - 1
    ip64, ix64 = O.i64(ip), O.i64(ix)
    A = mat(ip, ix, v)
    x = np.random.default_rng(4).normal(size=n)
    want = np.zeros(n)
    O.lib().mp_mat_mult(a(x), a(want), a(ip64), a(ix64), a(v), n)
    np.testing.assert_array_equal(A.mult(vec(x)).getArray(), want)


def test_spmv_rectangular_and_long_rows():
    rng = np.random.default_rng(3)
    d = rng.normal(size=(300, 5000)) * (rng.random((300, 5000)) < 0.6)
    ip, ix, v = dense_to_csr(d)
    A = mat(ip, ix, v, ncols=5000)
    x = rng.normal(size=5000)
    np.testing.assert_allclose(A.mult(vec(x)).getArray(), d @ x, rtol=1e-12, atol=1e-12)
    xt = rng.normal(size=300)
    np.testing.assert_allclose(A.multTranspose(vec(xt)).getArray(), d.T @ xt, rtol=1e-12,
                               atol=1e-11)


def test_spmv_transpose_follows_value_changes():
    """The transpose multiply runs over a cached copy of A^T's values: it
    must follow a change of A's values, and stay bit-identical to the
    reference's scatter for long columns too (the row-stream form of A^T)."""
    rng = np.random.default_rng(4)
    n = 400
    d = rng.normal(size=(n, n)) * (rng.random((n, n)) < 0.02)
    d[:, 7] = rng.normal(size=n)  # a full column: a 400-entry row of A^T
    np.fill_diagonal(d, 4.0)
    ip, ix, v = dense_to_csr(d)
    A = mat(ip, ix, v)
    x = rng.normal(size=n)

    def want(vals):
        out = np.zeros(n)
        O.lib().mp_mat_mult_transpose(a(x), a(out), a(O.i64(ip)), a(O.i64(ix)),
                                      a(np.ascontiguousarray(vals)), n, n)
        return out

    np.testing.assert_array_equal(A.multTranspose(vec(x)).getArray(), want(v))
    A.scale(1.5)
    np.testing.assert_array_equal(A.multTranspose(vec(x)).getArray(), want(v * 1.5))


def test_empty_matrix_and_vectors():
    A = mat(np.zeros(1, dtype=np.int64), np.zeros(0, dtype=np.int64), np.zeros(0))
    y = A.mult(PETSc.Vec().createSeq(0))
    assert y.getSize() == 0
    v = PETSc.Vec().createSeq(0)
    assert v.norm() == 0.0 and v.dot(v) == 0.0 and v.sum() == 0.0


@pytest.mark.parametrize("n", [1, 7, 16, 255, 256, 257, 4099, 100003])
def test_vec_maps_bit_exact_and_reductions(n):
    rng = np.random.default_rng(n)
    x, y, z = rng.normal(size=n), rng.normal(size=n), rng.normal(size=n)
    L = O.lib()
    cases = [
        ("axpy", lambda V, X, Y: V.axpy(2.5, X), lambda w: L.mp_vec_axpy(a(w), 2.5, a(x), n)),
        ("aypx", lambda V, X, Y: V.aypx(-1.5, X), lambda w: L.mp_vec_aypx(a(w), -1.5, a(x), n)),
        ("aypx0", lambda V, X, Y: V.aypx(0.0, X), lambda w: L.mp_vec_aypx(a(w), 0.0, a(x), n)),
        ("axpby", lambda V, X, Y: V.axpby(0.5, -3.0, X),
         lambda w: L.mp_vec_axpby(a(w), 0.5, -3.0, a(x), n)),
        ("axpbypcz", lambda V, X, Y: V.axpbypcz(1.5, -2.0, 0.25, X, Y),
         lambda w: L.mp_vec_axpbypcz(a(w), 1.5, -2.0, 0.25, a(x), a(y), n)),
        ("waxpy", lambda V, X, Y: V.waxpy(-0.75, X, Y),
         lambda w: L.mp_vec_waxpy(a(w), -0.75, a(x), a(y), n)),
        ("pmult", lambda V, X, Y: V.pointwiseMult(X, Y),
         lambda w: L.mp_vec_pointwise_mult(a(w), a(x), a(y), n)),
        ("pdiv", lambda V, X, Y: V.pointwiseDivide(X, Y),
         lambda w: L.mp_vec_pointwise_divide(a(w), a(x), a(y), n)),
        ("scale", lambda V, X, Y: V.scale(3.25), lambda w: L.mp_vec_scale(a(w), 3.25, n)),
        ("shift", lambda V, X, Y: V.shift(-1.0), lambda w: L.mp_vec_shift(a(w), -1.0, n)),
        ("recip", lambda V, X, Y: V.reciprocal(), lambda w: L.mp_vec_reciprocal(a(w), n)),
        ("abs", lambda V, X, Y: V.abs(), lambda w: L.mp_vec_abs(a(w), n)),
        ("sqrtabs", lambda V, X, Y: V.sqrtabs(), lambda w: L.mp_vec_sqrtabs(a(w), n)),
        ("chop", lambda V, X, Y: V.chop(0.5), lambda w: L.mp_vec_chop(a(w), n, 0.5)),
    ]
    for name, gpu, cpu in cases:
        V = vec(z)
        gpu(V, vec(x), vec(y))
        want = z.copy()
        cpu(want)
        np.testing.assert_array_equal(V.getArray(), want, err_msg=name)
    X, Y = vec(x), vec(y)
    # the ordered arithmetic sums in the reference's blocked order: equal to
    # the oracle's reductions to the last bit
    out, out2 = np.zeros(2), np.zeros(1)
    L.mp_vec_dot(a(x), a(y), a(out), n)
    assert X.dot(Y) == out[0]
    L.mp_vec_norm(a(x), 1, a(out), n)
    assert X.norm() == out[0]
    L.mp_vec_norm(a(x), 0, a(out), n)
    assert X.norm(PETSc.NormType.NORM_1) == out[0]
    L.mp_vec_sum(a(x), a(out), n)
    assert X.sum() == out[0]
    L.mp_vec_dot_norm2(a(x), a(y), a(out), a(out2), n)
    assert X.dotNorm2(Y) == (out[0], out2[0])
    assert X.dot(Y) == pytest.approx(float(x @ y), rel=1e-13, abs=1e-13)
    assert X.norm() == pytest.approx(float(np.linalg.norm(x)), rel=1e-13)
    assert X.norm(PETSc.NormType.NORM_1) == pytest.approx(float(np.abs(x).sum()), rel=1e-13)
    assert X.norm(PETSc.NormType.NORM_INFINITY) == float(np.abs(x).max())
    assert X.sum() == pytest.approx(float(x.sum()), rel=1e-11, abs=1e-11)
    d, q = X.dotNorm2(Y)
    assert d == pytest.approx(float(x @ y), rel=1e-13, abs=1e-13)
    assert q == pytest.approx(float(x @ x), rel=1e-13)
    assert X.max() == (int(np.argmax(x)), float(x.max()))
    assert X.min() == (int(np.argmin(x)), float(x.min()))
    M = vec(x)
    nrm = M.normalize()
    np.testing.assert_array_equal(M.getArray(), x / nrm)
    W = vec(np.zeros(n))
    W.maxpy([0.5, -2.0], [X, Y])
    np.testing.assert_array_equal(W.getArray(), (0.0 + 0.5 * x) + -2.0 * y)


def test_min_max_first_index_and_nan_rules():
    v = vec([3.0, 7.0, 7.0, -1.0, -1.0])
    assert v.max() == (1, 7.0) and v.min() == (3, -1.0)
    w = vec([1.0, np.nan, 5.0])
    assert w.max() == (2, 5.0)
    u = vec([np.nan, 1.0, 5.0])
    i, val = u.max()
    assert i == 0 and np.isnan(val)
    assert np.isnan(vec([1.0, np.nan, 3.0]).norm(PETSc.NormType.NORM_INFINITY))


def _pc(pt, A, **kw):
    pc = PETSc.PC().create()
    pc.setType(pt)
    for k, v in kw.items():
        getattr(pc, k)(v)
    pc.setOperators(A)
    pc.setUp()
    return pc


PCS = [
    ("jacobi", {}, {}),
    ("sor", {}, {}),
    ("sor", {"setSOROmega": 1.3, "setSORShift": 0.25}, {"omega": 1.3, "fshift": 0.25}),
    ("sor", {"setSORSymmetric": False}, {"symmetric": False}),
    ("ilu", {}, {}),
    ("ilu", {"setFactorLevels": 1}, {"levels": 1}),
    ("ilu", {"setFactorLevels": 2}, {"levels": 2}),
    ("ilu", {"setFactorOrdering": "rcm"}, {"ordering": "rcm"}),
    ("icc", {}, {}),
]


@pytest.mark.parametrize("levels", [1, 2])
def test_icc_levels_follow_the_level_of_fill_rule(levels):
    """IC(k) on a symmetric matrix has the upper triangle of ILU(k)'s pattern,
    and its apply solves with U^T D U.  (The reference's IC(k >= 1) symbolic
    merges the wrong row's staged columns, so this build is compared with the
    documented rule rather than with that output.)"""
    ip, ix, v = gallery.laplacian_2d(10)
    A = mat(ip, ix, v)
    icc = _pc("icc", A, setFactorLevels=levels)
    ilu = _pc("ilu", A, setFactorLevels=levels)
    fi, fl = icc._factor_arrays(), ilu._factor_arrays()
    n = 100
    for i in range(n):
        upper_ic = list(fi["bj"][fi["bi"][i]:fi["bdiag"][i]])
        upper_ilu = list(fl["bj"][fl["bdiag"][i + 1] + 1:fl["bdiag"][i]])
        assert upper_ic == upper_ilu
    M = icc.getFactorMatrix()._dense()
    x = np.random.default_rng(4).normal(size=n)
    y = PETSc.Vec().createSeq(n)
    icc.apply(vec(x), y)
    np.testing.assert_allclose(M @ y.getArray(), x, rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("pt,gopts,oopts", PCS)
@pytest.mark.parametrize("name", ["poisson3d_12", "convdiff_10", "dense_40"])
def test_pc_apply_bit_exact(pt, gopts, oopts, name):
    """Level-ordered ELL sweeps (at most 16 dependencies a row) and, for the
    dense case, the CSR sweep kernels that handle wider rows."""
    if name == "poisson3d_12":
        ip, ix, v = gallery.laplacian_3d(12)
    elif name == "dense_40":
        ip, ix, v = dense_to_csr(spd_dense(40, 11))
    else:
        if pt == "icc":
            pytest.skip("IC is for symmetric operators")
        ip, ix, v = gallery.convection_diffusion_3d(10)
    n = len(ip) - 1
    A = mat(ip, ix, v)
    pc = _pc(pt, A, **gopts)
    opc = O.OraclePC(pt, ip, ix, v, **oopts)
    x = np.random.default_rng(7).normal(size=n)
    y = PETSc.Vec().createSeq(n)
    pc.apply(vec(x), y)
    np.testing.assert_array_equal(y.getArray(), opc.apply(x))
    if pt in ("ilu", "icc"):
        f = pc._factor_arrays()
        np.testing.assert_array_equal(f["ba"][: len(opc.factor["ba"])], opc.factor["ba"])


def test_factor_matrix_reproduces_the_operator_for_exact_factors():
    d = tridiag_dense(20)
    A = PETSc.from_dense(d)
    for pt in ("ilu", "icc"):
        pc = _pc(pt, A)
        np.testing.assert_allclose(pc.getFactorMatrix()._dense(), d, rtol=1e-12, atol=1e-12)


def test_jacobi_variants_against_oracle():
    d = spd_dense(30, 4)
    d[3, 3] = -d[3, 3]
    ip, ix, v = dense_to_csr(d)
    A = mat(ip, ix, v)
    L = O.lib()
    ip64, ix64 = O.i64(ip), O.i64(ix)
    x = np.random.default_rng(9).normal(size=30)
    for jt in (0, 1, 2, 3):
        for useabs in (0, 1):
            pc = _pc("jacobi", A, setJacobiType=jt, setJacobiUseAbs=bool(useabs),
                     setJacobiRowl1Scale=0.5)
            y = PETSc.Vec().createSeq(30)
            pc.apply(vec(x), y)
            diag, didx = np.zeros(30), np.zeros(30)
            L.mp_pc_jacobi_setup(a(diag), jt, useabs, 1, 0.5, a(ip64), a(ix64), a(v), 30, a(didx))
            np.testing.assert_array_equal(y.getArray(), x * diag)
            ys = PETSc.Vec().createSeq(30)
            pc.applySymmetricLeft(vec(x), ys)
            ds = np.zeros(30)
            L.mp_pc_jacobi_setup_symmetric(a(ds), jt, a(ip64), a(ix64), a(v), 30)
            np.testing.assert_array_equal(ys.getArray(), x * ds)
