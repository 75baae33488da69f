"""Mixed precision (mojopetsc4py.mixed): FP32 inner FGMRES + ILU(0) inside FP64
refinement reaches rtol on the true FP64 residual, with the inexact (Jacobi
pass) and the exact (level-scheduled) triangle application, and agrees with
the plain FP64 GMRES + ILU(0) solution."""
import numpy as np
import pytest

from mojopetsc4py import PETSc, gallery

pytestmark = pytest.mark.gpu


def mat(ip, ix, v):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    return A


def true_relres(ip, ix, v, x, b):
    rows = np.repeat(np.arange(len(ip) - 1), np.diff(ip))
    ax = np.bincount(rows, weights=v * x[ix], minlength=len(ip) - 1)
    return np.linalg.norm(b - ax) / np.linalg.norm(b)


@pytest.mark.parametrize("tri_sweeps", [4, 0])
def test_refined_solution_meets_rtol_on_the_true_residual(tri_sweeps):
    from mojopetsc4py.mixed import MixedSolver

    ip, ix, v = gallery.convection_diffusion_3d(24)
    n = len(ip) - 1
    b = np.random.default_rng(7).uniform(-1, 1, n)
    A = mat(ip, ix, v)
    x = PETSc.Vec().createSeq(n)
    info = MixedSolver(A).solve(PETSc.Vec().createWithArray(b), x, rtol=1e-10,
                                tri_sweeps=tri_sweeps)
    assert info["converged"] and info["relres"] <= 1e-10
    assert info["passes"] >= 2
    xs = x.getArray()
    assert true_relres(ip, ix, v, xs, b) <= 1.05e-10
    # the plain FP64 path to the same tolerance
    ksp = PETSc.KSP().create()
    ksp.setOperators(A)
    ksp.setType("gmres")
    ksp.getPC().setType("ilu")
    ksp.setTolerances(rtol=1e-12, max_it=20000)
    xp = PETSc.Vec().createSeq(n)
    ksp.solve(PETSc.Vec().createWithArray(b), xp)
    assert np.linalg.norm(xs - xp.getArray()) <= 1e-8 * np.linalg.norm(xp.getArray())


def test_zero_rhs_and_size_checks():
    from mojopetsc4py.mixed import MixedSolver

    ip, ix, v = gallery.convection_diffusion_3d(6)
    n = len(ip) - 1
    A = mat(ip, ix, v)
    s = MixedSolver(A)
    x = PETSc.Vec().createWithArray(np.full(n, 3.0))
    info = s.solve(PETSc.Vec().createSeq(n), x)
    assert info["converged"] and info["passes"] == 0
    assert np.all(x.getArray() == 0.0)
    with pytest.raises(ValueError):
        s.solve(PETSc.Vec().createSeq(n + 1), x)
