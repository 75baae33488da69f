"""Batched CG (mojopetsc4py.batch): every (system, column) pair against the
single-system device CG on the same matrix and right-hand side, the reported
residuals against an FP64 residual computed here, the FP32-inner refinement
form against rtol on the true residual, and run-to-run determinism."""
import numpy as np
import pytest

from mojopetsc4py import PETSc, gallery

pytestmark = pytest.mark.gpu


def systems(sizes, seed=11):
    rng = np.random.default_rng(seed)
    return [gallery.rgg_laplacian(n, rng) for n in sizes]


def residual(sysm, X, B):
    """||b - A x|| / ||b|| per pair, in FP64 on the host."""
    out = []
    r0 = 0
    for ip, ix, v in sysm:
        n = len(ip) - 1
        rows = np.repeat(np.arange(n), np.diff(ip))
        x = X[r0:r0 + n]
        ax = np.zeros_like(x)
        np.add.at(ax, rows, v[:, None] * x[ix])
        b = B[r0:r0 + n]
        out.append(np.linalg.norm(b - ax, axis=0) / np.maximum(np.linalg.norm(b, axis=0), 1e-300))
        r0 += n
    return np.array(out)


def single_cg(ip, ix, v, b, pc, rtol):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    ksp = PETSc.KSP().create()
    ksp.setOperators(A)
    ksp.setType("cg")
    ksp.getPC().setType(pc)
    ksp.setTolerances(rtol=rtol, atol=1e-50, max_it=10000)
    x = PETSc.Vec().createSeq(n)
    ksp.solve(PETSc.Vec().createWithArray(b), x)
    return x.getArray().copy(), ksp.getIterationNumber(), ksp.getConvergedReason()


@pytest.mark.parametrize("nrhs,pc", [(4, "jacobi"), (1, "none"), (16, "jacobi")])
def test_each_pair_follows_the_single_system_cg(nrhs, pc):
    from mojopetsc4py.batch import BatchedCG

    sysm = systems([300, 1200, 57, 2500, 800])
    solver = BatchedCG(sysm, nrhs=nrhs)
    n = sum(len(ip) - 1 for ip, _, _ in sysm)
    B = np.random.default_rng(5).normal(size=(n, nrhs))
    X, info = solver.solve(B, pc=pc, rtol=1e-10)
    r0 = 0
    for s, (ip, ix, v) in enumerate(sysm):
        m = len(ip) - 1
        for c in range(nrhs):
            x1, its1, reason1 = single_cg(ip, ix, v, B[r0:r0 + m, c].copy(), pc, 1e-10)
            assert info["reason"][s, c] == reason1 == 2
            # same recurrence; the batched kernels fuse multiply-adds and sum
            # in another order, so the count moves by rounding on the
            # ill-conditioned graphs (a few iterations in hundreds)
            slack = max(2, int(0.02 * its1))
            assert abs(int(info["its"][s, c]) - its1) <= slack, (s, c, info["its"][s, c], its1)
            xb = X[r0:r0 + m, c]
            assert np.linalg.norm(xb - x1) <= 1e-7 * np.linalg.norm(x1)
        r0 += m
    # the residual of a converged iterate is itself evaluated to ~1e-15
    np.testing.assert_allclose(info["relres"], residual(sysm, X, B), rtol=1e-4, atol=1e-14)


def test_fp32_inner_refinement_meets_rtol_on_the_true_residual():
    from mojopetsc4py.batch import BatchedCG

    sysm = systems([700, 4000, 1500, 90, 2600, 3100], seed=3)
    n = sum(len(ip) - 1 for ip, _, _ in sysm)
    solver = BatchedCG(sysm, nrhs=16)
    B = np.random.default_rng(9).normal(size=(n, 16))
    B[:, 3] = 0.0  # a zero right-hand side converges at once with x = 0
    X, info = solver.solve(B, pc="jacobi", precision="fp32", rtol=1e-10)
    true = residual(sysm, X, B)
    mask = np.ones_like(true, dtype=bool)
    mask[:, 3] = False
    assert np.all(true[mask] <= 1e-10 * 1.01), true.max()
    assert np.all(info["reason"] == 2)
    assert np.all(X[:, 3] == 0.0)
    assert info["passes"] >= 2
    np.testing.assert_allclose(info["relres"][mask], true[mask], rtol=1e-4, atol=1e-14)


def test_solves_are_deterministic_and_the_tuner_reports_its_choice():
    import torch
    from mojopetsc4py.batch import BatchedCG

    sysm = systems([1000, 2000, 3000], seed=7)
    n = sum(len(ip) - 1 for ip, _, _ in sysm)
    solver = BatchedCG(sysm, nrhs=8)
    t = solver.tuning
    assert t["block"] in (128, 256, 512) and t["columns_per_thread"] in (1, 2, 4)
    assert t["tile_rows"] in (128, 512) and t["spmm_us"] > 0
    B = torch.randn(n, 8, dtype=torch.float64, device="cuda")
    X1, i1 = solver.solve(B, rtol=1e-9)
    X1 = X1.clone()
    X2, i2 = solver.solve(B, rtol=1e-9)
    assert torch.equal(X1, X2)
    assert np.array_equal(i1["its"], i2["its"])


@pytest.mark.parametrize("pc", ["jacobi", "icc"])
def test_each_pair_matches_the_oracle(pc, monkeypatch):
    """Every (system, column) pair against the oracle's CG on the same system
    and right-hand side (the systems keep the caller's row numbering, so the
    IC(0) factor is the oracle's).  The batched kernels fold with fused
    multiply-adds and sum the dots in tile order, so the iteration count may
    move by rounding on these ill-conditioned graphs; the iterate agrees to
    the solve's accuracy."""
    import oracle as O
    from mojopetsc4py.batch import BatchedCG

    monkeypatch.setenv("GPETSC_BATCH_RCM", "0")
    sysm = systems([300, 1200, 57, 900], seed=21)
    solver = BatchedCG(sysm, nrhs=4)
    n = sum(len(ip) - 1 for ip, _, _ in sysm)
    B = np.random.default_rng(6).normal(size=(n, 4))
    X, info = solver.solve(B, pc=pc, rtol=1e-10)
    r0 = 0
    for s, (ip, ix, v) in enumerate(sysm):
        m = len(ip) - 1
        for c in range(4):
            ref = O.solve("cg", ip, ix, v, B[r0:r0 + m, c].copy(), pc_type=pc, rtol=1e-10,
                          atol=1e-50, divtol=1e4, max_it=10000)
            assert info["reason"][s, c] == ref["reason"] == 2
            slack = max(2, int(0.02 * ref["its"]))
            assert abs(int(info["its"][s, c]) - ref["its"]) <= slack, (s, c, info["its"][s, c],
                                                                       ref["its"])
            xr = ref["x"]
            assert np.linalg.norm(X[r0:r0 + m, c] - xr) <= 1e-7 * np.linalg.norm(xr)
        r0 += m


def test_icc_batches_converge_in_fewer_iterations_than_jacobi():
    """IC(0) in the default (RCM-renumbered) rows: every pair meets rtol on
    its true residual, matches a dense solve, and needs fewer iterations
    than Jacobi on the same pairs."""
    from mojopetsc4py.batch import BatchedCG

    sysm = systems([500, 1800, 90, 2400], seed=5)
    n = sum(len(ip) - 1 for ip, _, _ in sysm)
    solver = BatchedCG(sysm, nrhs=16)
    B = np.random.default_rng(8).normal(size=(n, 16))
    Xi, ii = solver.solve(B, pc="icc", rtol=1e-10)
    _, ij = solver.solve(B, pc="jacobi", rtol=1e-10)
    assert np.all(ii["reason"] == 2)
    assert np.all(residual(sysm, Xi, B) <= 1e-8)
    assert ii["its"].mean() < 0.8 * ij["its"].mean()
    r0 = 0
    for ip, ix, v in sysm:
        m = len(ip) - 1
        dense = np.zeros((m, m))
        dense[np.repeat(np.arange(m), np.diff(ip)), ix] = v
        want = np.linalg.solve(dense, B[r0:r0 + m])
        np.testing.assert_allclose(Xi[r0:r0 + m], want, rtol=0,
                                   atol=1e-7 * np.abs(want).max())
        r0 += m
    with pytest.raises(Exception):
        solver.solve(B, pc="icc", precision="fp32", rtol=1e-8)
