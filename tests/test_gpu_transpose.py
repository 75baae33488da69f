"""The transposed preconditioner apply and the transposed solve.

PC.applyTranspose keeps the reference's behaviour (the plain apply,
python/mojopetsc4py/PETSc/PC.py:635-642) unless setUseExactTranspose(True)
asks for the true transpose M^-T; KSP.solveTranspose solves A^T x = b with
the same operator and preconditioner (A^T multiplies, M^-T applies), as
upstream PETSc's KSPSolveTranspose does.  The reference has neither, so the
checks are mathematical: M^-T must be the transpose of M^-1 (dense on small
systems, the adjoint identity <M^-T x, z> = <x, M^-1 z> on larger ones), and
a transposed solve must solve A^T x = b.
"""
import numpy as np
import pytest

from helpers import dense_to_csr, nonsym_banded
from mojopetsc4py import PETSc, _lib, gallery
from mojopetsc4py._lib import GPError

pytestmark = pytest.mark.gpu


def _mat(ip, ix, v):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    return A


def _pc(pt, A, exact=True, **opts):
    pc = PETSc.PC().create()
    pc.setType(pt)
    for k, val in opts.items():
        getattr(pc, k)(val)
    pc.setOperators(A)
    pc.setUp()
    pc.setUseExactTranspose(exact)
    return pc


def _apply(fn, x):
    y = PETSc.Vec().createSeq(len(x))
    fn(PETSc.Vec().createWithArray(np.asarray(x, dtype=np.float64)), y)
    return y.getArray().copy()


def _dense(fn, n):
    return np.column_stack([_apply(fn, np.eye(n)[:, j]) for j in range(n)])


ILU_OPTS = [{}, {"setFactorLevels": 1}, {"setFactorOrdering": "rcm"}]


@pytest.mark.parametrize("opts", ILU_OPTS, ids=["ilu0", "ilu1", "ilu0-rcm"])
def test_ilu_transposed_apply_is_the_transpose(opts):
    a = nonsym_banded(60, 3)
    pc = _pc("ilu", _mat(*dense_to_csr(a)), **opts)
    minv = _dense(pc.apply, 60)
    mtinv = _dense(pc.applyTranspose, 60)
    np.testing.assert_allclose(mtinv, minv.T, rtol=1e-12, atol=1e-14 * np.abs(minv).max())
    # and it is not the plain apply on this nonsymmetric operator
    assert np.abs(mtinv - minv).max() > 1e-6 * np.abs(minv).max()


@pytest.mark.parametrize("name", ["convdiff_12", "advdiff_32"])
def test_ilu_transposed_apply_satisfies_the_adjoint_identity(name):
    if name == "convdiff_12":
        ip, ix, v = gallery.convection_diffusion_3d(12)
    else:
        kappa = np.exp(gallery.gaussian_random_field(32, np.random.default_rng(3), corr=8.0))
        ip, ix, v = gallery.advection_diffusion_2d(kappa, peclet=2.0)
    n = len(ip) - 1
    pc = _pc("ilu", _mat(ip, ix, v))
    rng = np.random.default_rng(4)
    for _ in range(3):
        x, z = rng.normal(size=n), rng.normal(size=n)
        lhs = _apply(pc.applyTranspose, x) @ z
        rhs = x @ _apply(pc.apply, z)
        assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + abs(rhs))


def test_default_apply_transpose_is_the_plain_apply():
    a = nonsym_banded(40, 2)
    pc = _pc("ilu", _mat(*dense_to_csr(a)), exact=False)
    x = np.random.default_rng(1).normal(size=40)
    np.testing.assert_array_equal(_apply(pc.applyTranspose, x), _apply(pc.apply, x))


@pytest.mark.parametrize("pt", ["none", "jacobi", "icc"])
def test_symmetric_preconditioners_transpose_to_themselves(pt):
    ip, ix, v = gallery.laplacian_2d(12)
    pc = _pc(pt, _mat(ip, ix, v))
    x = np.random.default_rng(2).normal(size=144)
    np.testing.assert_array_equal(_apply(pc.applyTranspose, x), _apply(pc.apply, x))


def test_sor_has_no_transposed_apply():
    a = nonsym_banded(30, 2)
    pc = _pc("sor", _mat(*dense_to_csr(a)))
    with pytest.raises(GPError):
        _apply(pc.applyTranspose, np.ones(30))


SOLVES = [("gmres", "ilu"), ("fgmres", "ilu"), ("bcgs", "ilu"), ("gmres", "jacobi"),
          ("cg", "icc")]


@pytest.mark.parametrize("kt,pt", SOLVES)
def test_solve_transpose_solves_the_transposed_system(kt, pt):
    if kt == "cg":
        ip, ix, v = gallery.laplacian_3d(10)
    else:
        ip, ix, v = gallery.convection_diffusion_3d(10)
    n = len(ip) - 1
    A = _mat(ip, ix, v)
    dense = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(ip))
    dense[rows, ix] = v
    b = np.random.default_rng(5).normal(size=n)
    ksp = PETSc.KSP().create()
    ksp.setOperators(A)
    ksp.setType(kt)
    ksp.getPC().setType(pt)
    ksp.setTolerances(rtol=1e-12, atol=1e-50, max_it=2000)
    want = np.linalg.solve(dense.T, b)
    for _ in range(2):  # the second solve reuses the captured graph
        x = PETSc.Vec().createSeq(n)
        ksp.solveTranspose(PETSc.Vec().createWithArray(b), x)
        assert ksp.getConvergedReason() > 0
        got = x.getArray()
        assert np.linalg.norm(b - dense.T @ got) <= 1e-9 * np.linalg.norm(b)
        assert np.linalg.norm(got - want) <= 1e-8 * np.linalg.norm(want)
    # and the same KSP still solves A x = b afterwards
    x = PETSc.Vec().createSeq(n)
    ksp.solve(PETSc.Vec().createWithArray(b), x)
    assert np.linalg.norm(b - dense @ x.getArray()) <= 1e-9 * np.linalg.norm(b)


FORMS = [("level-order", False, 0), ("chosen", True, 0), ("chunks-64", True, 64),
         ("chunks-333", True, 333)]


@pytest.fixture
def _restore_form():
    yield
    _lib.set_sweep_form(True, 0)


@pytest.mark.usefixtures("_restore_form")
@pytest.mark.parametrize("opts", ILU_OPTS, ids=["ilu0", "ilu1", "ilu0-rcm"])
def test_transposed_apply_is_the_same_in_every_sweep_form(opts):
    """The transposed sweeps (U^T, then L^T) take the chunked form where the
    set-up's schedule model prefers it, like the plain ones; every form gives
    the same bits."""
    kappa = np.exp(gallery.gaussian_random_field(24, np.random.default_rng(3), corr=6.0))
    ip, ix, v = gallery.advection_diffusion_2d(kappa, peclet=2.0)
    n = len(ip) - 1
    x = np.random.default_rng(8).normal(size=n)
    got = {}
    for name, tiles, rows in FORMS:
        _lib.set_sweep_form(tiles, rows)
        pc = _pc("ilu", _mat(ip, ix, v), **opts)
        got[name] = _apply(pc.applyTranspose, x)
        form = _lib.sweep_form(pc._handle(), transposed=True)
        if rows:
            assert form["first"]["tiled"] and form["second"]["tiled"], form
        if not tiles:
            assert not form["first"]["tiled"] and not form["second"]["tiled"], form
    for name in got:
        np.testing.assert_array_equal(got[name], got["level-order"], err_msg=name)
    # and it is still the transpose of the plain apply
    z = np.random.default_rng(9).normal(size=n)
    pc = _pc("ilu", _mat(ip, ix, v), **opts)
    lhs = got["chosen"] @ z
    rhs = x @ _apply(pc.apply, z)
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + abs(rhs))
