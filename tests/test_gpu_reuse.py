"""Solver objects reused across value changes, PC re-set-ups and new matrices.

A KSP keeps its captured solve graph while the operator, the PC set-up and the
options are unchanged.  These tests change each of them in turn and compare
the reused solver with a freshly built one on the same inputs: the results
must be identical to the bit.

* SOR's inverted diagonal and sweep coefficients are functions of the
  matrix values (the reference recomputes them on every apply,
  src/ported.mojo:610-633); here they are recomputed when the values
  changed, so a value change between solves must be seen.
* A PC set up again (new options) gets new device arrays; a matrix created
  after another was destroyed may get the same host address.  Cached graphs
  key on unique ids, so neither may replay a graph of the old objects.
"""
import numpy as np
import pytest

from mojopetsc4py import PETSc, gallery

pytestmark = pytest.mark.gpu


def _mat(ip, ix, v):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    return A


def _ksp(A, kt, pt, omega=None):
    ksp = PETSc.KSP().create()
    ksp.setOperators(A)
    ksp.setType(kt)
    ksp.getPC().setType(pt)
    if omega is not None:
        ksp.getPC().setSOROmega(omega)
    ksp.setTolerances(rtol=1e-10, atol=1e-50, max_it=500)
    return ksp


def _solve(ksp, b):
    x = PETSc.Vec().createSeq(len(b))
    ksp.solve(PETSc.Vec().createWithArray(b), x)
    return x.getArray().copy(), ksp.getIterationNumber(), ksp.getConvergedReason()


def _fresh(ip, ix, v, b, kt, pt, omega=None):
    return _solve(_ksp(_mat(ip, ix, v), kt, pt, omega), b)


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    assert a[1:] == b[1:]


@pytest.mark.parametrize("kt", ["bcgs", "gmres"])
def test_sor_follows_value_changes(kt):
    ip, ix, v = gallery.convection_diffusion_3d(10)
    b = np.random.default_rng(3).uniform(-1, 1, len(ip) - 1)
    A = _mat(ip, ix, v)
    ksp = _ksp(A, kt, "sor", 1.2)
    first = _solve(ksp, b)
    _same(first, _fresh(ip, ix, v, b, kt, "sor", 1.2))
    _same(_solve(ksp, b), first)  # unchanged values: the cached arrays serve
    rng = np.random.default_rng(4)
    for _ in range(2):
        # new values, same pattern (diagonally dominant again)
        v = v * rng.uniform(0.8, 1.25, len(v))
        A.setValuesCSR(ip, ix, v)
        A.assemble()
        _same(_solve(ksp, b), _fresh(ip, ix, v, b, kt, "sor", 1.2))


def test_sor_standalone_apply_follows_value_changes():
    ip, ix, v = gallery.laplacian_2d(20)
    n = len(ip) - 1
    x = PETSc.Vec().createWithArray(np.random.default_rng(5).normal(size=n))
    A = _mat(ip, ix, v)
    pc = PETSc.PC().create()
    pc.setType("sor")
    pc.setOperators(A)
    pc.setUp()
    y0 = PETSc.Vec().createSeq(n)
    pc.apply(x, y0)
    A.scale(2.0)
    y1 = PETSc.Vec().createSeq(n)
    pc.apply(x, y1)
    ref = PETSc.PC().create()
    ref.setType("sor")
    ref.setOperators(_mat(ip, ix, 2.0 * v))
    ref.setUp()
    y2 = PETSc.Vec().createSeq(n)
    ref.apply(x, y2)
    np.testing.assert_array_equal(y1.getArray(), y2.getArray())
    assert not np.array_equal(y0.getArray(), y1.getArray())


def test_pc_set_up_again_recaptures_the_solve():
    ip, ix, v = gallery.convection_diffusion_3d(9)
    b = np.random.default_rng(6).uniform(-1, 1, len(ip) - 1)
    ksp = _ksp(_mat(ip, ix, v), "bcgs", "sor", 1.0)
    _same(_solve(ksp, b), _fresh(ip, ix, v, b, "bcgs", "sor", 1.0))
    for omega in (1.5, 0.8):
        ksp.getPC().setSOROmega(omega)  # the PC is set up again on the next solve
        _same(_solve(ksp, b), _fresh(ip, ix, v, b, "bcgs", "sor", omega))


@pytest.mark.parametrize("pt", ["ilu", "jacobi", "sor"])
def test_new_matrices_never_replay_an_old_graph(pt):
    """Matrices of different values created and destroyed in turn: the host
    allocator hands out recycled addresses, the solve must follow the new
    matrix every time."""
    ip, ix, v0 = gallery.convection_diffusion_3d(8)
    b = np.random.default_rng(7).uniform(-1, 1, len(ip) - 1)
    ksp = PETSc.KSP().create()
    ksp.setType("gmres")
    ksp.getPC().setType(pt)
    ksp.setTolerances(rtol=1e-10, atol=1e-50, max_it=500)
    rng = np.random.default_rng(8)
    for k in range(4):
        v = v0 * rng.uniform(0.8, 1.25, len(v0))
        A = _mat(ip, ix, v)
        ksp.setOperators(A)
        _same(_solve(ksp, b), _fresh(ip, ix, v, b, "gmres", pt))
        A.destroy()
        del A
