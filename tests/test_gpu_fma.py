"""The fused multiply-add arithmetic (the default): kernels fold each product
into an FMA in the reference's order, so results differ from the exact form
(which the parity suites check bit for bit) by rounding only.  These tests
bound that difference: SpMV entrywise against the exact bound, PC applies
against the oracle, and whole solves by iteration count and iterate."""
import numpy as np
import pytest

import oracle as O
from helpers import dense_to_csr, nonsym_banded, spd_dense
from mojopetsc4py import PETSc, gallery

pytestmark = [pytest.mark.gpu, pytest.mark.fma]

EPS = np.finfo(np.float64).eps


def mat(ip, ix, v):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    return A


def vec(x):
    return PETSc.Vec().createWithArray(np.asarray(x, dtype=np.float64))


def oracle_spmv(ip, ix, v, x):
    ip64, ix64 = O.i64(ip), O.i64(ix)
    v, x = O.f64(v), O.f64(x)
    y = np.zeros(len(ip) - 1)
    O.lib().mp_mat_mult(O.a(x), O.a(y), O.a(ip64), O.a(ix64), O.a(v), len(ip) - 1)
    return y


def test_arithmetic_switch_round_trip():
    import mojopetsc4py

    assert mojopetsc4py.get_arithmetic() == "fma"
    for mode in ("exact", "ordered", "fma"):
        mojopetsc4py.set_arithmetic(mode)
        assert mojopetsc4py.get_arithmetic() == mode
    with pytest.raises(ValueError):
        mojopetsc4py.set_arithmetic("fast")


@pytest.mark.parametrize("name", ["poisson3d_24", "convdiff_12", "nonsym_300"])
def test_spmv_within_the_rounding_bound(name):
    ip, ix, v = {
        "poisson3d_24": lambda: gallery.laplacian_3d(24),
        "convdiff_12": lambda: gallery.convection_diffusion_3d(12),
        "nonsym_300": lambda: dense_to_csr(nonsym_banded(300, 5)),
    }[name]()
    n = len(ip) - 1
    A = mat(ip, ix, v)
    x = np.random.default_rng(1).normal(size=n)
    y = PETSc.Vec().createSeq(n)
    A.mult(vec(x), y)
    ref = oracle_spmv(ip, ix, v, x)
    # |fl(sum) - sum| <= k eps sum |a_ij x_j| for a k-term sum, either form
    absrow = oracle_spmv(ip, ix, np.abs(v), np.abs(x))
    k = np.diff(ip).max()
    assert np.all(np.abs(y.getArray() - ref) <= 2 * k * EPS * absrow + 1e-300)


@pytest.mark.parametrize("pt", ["jacobi", "sor", "ilu", "icc"])
def test_pc_apply_close_to_the_oracle(pt):
    ip, ix, v = gallery.laplacian_3d(12)
    n = len(ip) - 1
    A = mat(ip, ix, v)
    pc = PETSc.PC().create()
    pc.setType(pt)
    pc.setOperators(A)
    pc.setUp()
    opc = O.OraclePC(pt, ip, ix, v)
    x = np.random.default_rng(7).normal(size=n)
    y = PETSc.Vec().createSeq(n)
    pc.apply(vec(x), y)
    ref = opc.apply(x)
    assert np.linalg.norm(y.getArray() - ref) <= 1e-12 * np.linalg.norm(ref)


SOLVES = [
    ("cg", "none", "poisson3d_16", 2),
    ("cg", "jacobi", "poisson3d_16", 2),
    ("cg", "icc", "poisson3d_16", 2),
    ("gmres", "ilu", "convdiff_12", 2),
    ("fgmres", "ilu", "convdiff_12", 2),
    ("bcgs", "sor", "convdiff_12", 20),
]


@pytest.mark.parametrize("kt,pt,name,slack", SOLVES)
def test_solve_matches_the_oracle_to_rounding(kt, pt, name, slack):
    if name == "poisson3d_16":
        ip, ix, v = gallery.laplacian_3d(16)
    else:
        ip, ix, v = gallery.convection_diffusion_3d(12)
    n = len(ip) - 1
    b = np.random.default_rng(3).normal(size=n)
    ref = O.solve(kt, ip, ix, v, b, pc_type=pt, rtol=1e-10, max_it=2000)
    A = mat(ip, ix, v)
    ksp = PETSc.KSP().create()
    ksp.setOperators(A)
    ksp.setType(kt)
    ksp.getPC().setType(pt)
    ksp.setTolerances(rtol=1e-10, max_it=2000)
    x = PETSc.Vec().createSeq(n)
    ksp.solve(vec(b), x)
    assert ksp.getConvergedReason() == ref["reason"]
    assert abs(ksp.getIterationNumber() - ref["its"]) <= slack
    xr = ref["x"]
    assert np.linalg.norm(x.getArray() - xr) <= 1e-8 * np.linalg.norm(xr)
