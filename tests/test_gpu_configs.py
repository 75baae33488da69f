"""The benchmark workloads at their stated sizes, against the oracle.

Each case is one plain FP64 solve of a configuration the benchmark names:

  C1  2-D 5-point Poisson 128^2, b = ones, x0 = 0: CG + ILU(0) and
      GMRES(30) + Jacobi, rtol 1e-12, max_it 500
  C2  3-D 7-point Poisson 128^3, b uniform[-1, 1] (seed 5): CG + Jacobi,
      CG + ICC(0), GMRES(30) + ILU(0), BiCGStab + SOR(omega 1.2, symmetric
      sweep), rtol 1e-10, max_it 10000
  C3  3-D upwind convection-diffusion 96^3 (cell Peclet 10), b uniform
      (seed 7): GMRES(30) + ILU(0), rtol 1e-10
  C5  2-D advection-diffusion 256^2, kappa = exp(GRF) (seed 13), Peclet 2,
      b = ones: GMRES(30) + ILU(0), rtol 1e-10
  the reference's published GMRES / FGMRES 128^2 cases (b normal, seed 5,
      rtol 1e-10, max_it 2000: 2000 iterations, CONVERGED_ITS)

Two arithmetics are checked against the same oracle result:

* fma (the default, the one bench.py times): the same converged reason, the
  same iteration count for CG / GMRES / FGMRES and the iterate within 1e-10
  relative; BiCGStab within 2 iterations and 1e-8.
* ordered (every reduction in the reference's blocked order): the solve is
  bit-identical to the oracle's -- iteration count, iterate and residual
  history.

The oracle solves of the large cases take seconds to tens of seconds on one
core; they are started together on a thread pool when the module is first
used (the oracle's C calls release the GIL), so they overlap each other and
the GPU solves.
"""
import functools
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle as O
from mojopetsc4py import PETSc, gallery

pytestmark = pytest.mark.gpu

T12 = dict(rtol=1e-12, atol=1e-50, divtol=1e30, max_it=500)
T10 = dict(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=10000)
TP = dict(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=2000)


@functools.lru_cache(maxsize=None)
def problem(key):
    if key == "lap2d_128":
        return gallery.laplacian_2d(128)
    if key == "lap3d_128":
        return gallery.laplacian_3d(128)
    if key == "convdiff_96":
        return gallery.convection_diffusion_3d(96)
    if key == "advdiff_256":
        rng = np.random.default_rng(13)
        kappa = np.exp(gallery.gaussian_random_field(256, rng, corr=16.0))
        return gallery.advection_diffusion_2d(kappa, peclet=2.0)
    raise KeyError(key)


@functools.lru_cache(maxsize=None)
def rhs(key):
    if key == "ones_16384":
        return np.ones(16384)
    if key == "ones_65536":
        return np.ones(65536)
    if key == "normal5_16384":
        return np.random.default_rng(5).normal(size=16384)
    if key == "uniform5_128^3":
        return np.random.default_rng(5).uniform(-1.0, 1.0, 128 ** 3)
    if key == "uniform7_96^3":
        return np.random.default_rng(7).uniform(-1.0, 1.0, 96 ** 3)
    raise KeyError(key)


# name -> (matrix, rhs, ksp type, pc type, pc options, tolerances)
CASES = {
    "C1 cg+ilu(0)": ("lap2d_128", "ones_16384", "cg", "ilu", {}, T12),
    "C1 gmres(30)+jacobi": ("lap2d_128", "ones_16384", "gmres", "jacobi", {}, T12),
    "C2 cg+jacobi": ("lap3d_128", "uniform5_128^3", "cg", "jacobi", {}, T10),
    "C2 cg+icc(0)": ("lap3d_128", "uniform5_128^3", "cg", "icc", {}, T10),
    "C2 gmres(30)+ilu(0)": ("lap3d_128", "uniform5_128^3", "gmres", "ilu", {}, T10),
    "C2 bcgs+sor(1.2)": ("lap3d_128", "uniform5_128^3", "bcgs", "sor", {"omega": 1.2}, T10),
    "C3 gmres(30)+ilu(0)": ("convdiff_96", "uniform7_96^3", "gmres", "ilu", {}, T10),
    "C5 gmres(30)+ilu(0)": ("advdiff_256", "ones_65536", "gmres", "ilu", {}, T10),
    "published gmres+none 128^2": ("lap2d_128", "normal5_16384", "gmres", "none", {}, TP),
    "published fgmres+none 128^2": ("lap2d_128", "normal5_16384", "fgmres", "none", {}, TP),
}

_pool = None
_futures = {}


def _oracle(name):
    mk, bk, kt, pt, po, tol = CASES[name]
    ip, ix, v = problem(mk)
    return O.solve(kt, ip, ix, v, rhs(bk), pc_type=pt, **tol, **po)


def oracle_result(name):
    global _pool
    if _pool is None:
        # build every input first (numpy, GIL-bound), then run all oracle
        # solves at once
        for mk, bk, *_ in CASES.values():
            problem(mk)
            rhs(bk)
        _pool = ThreadPoolExecutor(max_workers=len(CASES))
        for nm in CASES:
            _futures[nm] = _pool.submit(_oracle, nm)
    return _futures[name].result()


def gpu_solve(name):
    mk, bk, kt, pt, po, tol = CASES[name]
    ip, ix, v = problem(mk)
    b = rhs(bk)
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    pc = PETSc.PC().create()
    pc.setType(pt)
    if "omega" in po:
        pc.setSOROmega(po["omega"])
    pc.setOperators(A)
    ksp = PETSc.KSP().create()
    ksp.setPC(pc)
    ksp.setType(kt)
    ksp.setOperators(A)
    ksp.setTolerances(**tol)
    if kt in ("gmres", "fgmres"):
        ksp.setGMRESRestart(30)
    ksp.setConvergenceHistory()
    xv = PETSc.Vec().createSeq(n)
    ksp.solve(PETSc.Vec().createWithArray(b), xv)
    return {"x": xv.getArray().copy(), "its": ksp.getIterationNumber(),
            "reason": ksp.getConvergedReason(),
            "history": ksp.getConvergenceHistory().copy()}


@pytest.mark.fma
@pytest.mark.parametrize("name", list(CASES))
def test_config_in_the_timed_arithmetic(name):
    kt = CASES[name][2]
    r = oracle_result(name)
    g = gpu_solve(name)
    assert g["reason"] == r["reason"], (g["reason"], r["reason"])
    rel = np.linalg.norm(g["x"] - r["x"]) / np.linalg.norm(r["x"])
    if kt == "bcgs":
        assert abs(g["its"] - r["its"]) <= 2, (g["its"], r["its"])
        assert rel <= 1e-8, rel
    else:
        assert g["its"] == r["its"], (g["its"], r["its"])
        assert rel <= 1e-10, rel


@pytest.mark.parametrize("name", list(CASES))
def test_config_bit_identical_in_the_ordered_arithmetic(name):
    r = oracle_result(name)
    g = gpu_solve(name)
    assert (g["its"], g["reason"]) == (r["its"], r["reason"])
    np.testing.assert_array_equal(g["x"], r["x"])
    np.testing.assert_array_equal(g["history"][: g["its"] + 1], r["history"])
