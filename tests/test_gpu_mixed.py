"""Mixed precision (mojopetsc4py.mixed): FP32 inner FGMRES + ILU(0) inside FP64
refinement reaches rtol on the true FP64 residual, with every form of the
triangle application (point-Jacobi passes, block passes, the exact
level-scheduled sweeps, the multicolour factor), and agrees with the plain
FP64 GMRES + ILU(0) solution."""
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


# (passes per triangle, block rows, ordering): point-Jacobi passes, block
# passes (chosen and forced run lengths, one cutting grid lines), the exact
# FP64 sweeps, and the multicolour factor (one pass is exact for two colours)
FORMS = [(4, 0, "natural"), (2, -1, "natural"), (2, 100, "natural"), (0, 0, "natural"),
         (1, 0, "multicolor")]


@pytest.mark.parametrize("tri_sweeps,tri_block,ordering", FORMS)
def test_refined_solution_meets_rtol_on_the_true_residual(tri_sweeps, tri_block, ordering):
    from mojopetsc4py.mixed import MixedSolver

    ip, ix, v = gallery.convection_diffusion_3d(24)
    n = len(ip) - 1
    b = np.random.default_rng(7).uniform(-1, 1, n)
    A = mat(ip, ix, v)
    x = PETSc.Vec().createSeq(n)
    info = MixedSolver(A, ordering=ordering).solve(PETSc.Vec().createWithArray(b), x,
                                                   rtol=1e-10, tri_sweeps=tri_sweeps,
                                                   tri_block=tri_block)
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


def test_multicolour_passes_apply_the_triangles_exactly():
    """With two colours one pass per triangle is the exact triangular solve:
    the inner iteration counts match those of the exact FP64 sweeps."""
    from mojopetsc4py.mixed import MixedSolver

    ip, ix, v = gallery.convection_diffusion_3d(16)
    n = len(ip) - 1
    b = np.random.default_rng(3).uniform(-1, 1, n)
    A = mat(ip, ix, v)
    s = MixedSolver(A, ordering="multicolor")
    x = PETSc.Vec().createSeq(n)
    one = s.solve(PETSc.Vec().createWithArray(b), x, rtol=1e-10, tri_sweeps=1)
    exact = s.solve(PETSc.Vec().createWithArray(b), x, rtol=1e-10, tri_sweeps=0)
    assert one["converged"] and exact["converged"]
    assert abs(one["inner_its"] - exact["inner_its"]) <= 2
