"""The three forms of the ILU / IC / SOR triangular sweeps against the oracle.

The level-ordered form hands out rows in dependency-level order, 32 to a
warp; the chunked form gives runs of consecutive rows to one CTA, whose
compute warp walks the chunk level by level with in-chunk values in shared
memory while its fetch warps poll the values of earlier chunks; the brick
form (grid-structured sweeps in natural order) gives a brick of grid lines of
one plane to one CTA, one line a thread, with the neighbouring line's values
in shared memory and the faces of other bricks fetched from L2 into a
shared-memory ring.  All must
reproduce the reference's sequential sweeps bit for bit in the exact
arithmetic, whatever the chunk size: chunk sizes that cut grid lines (so a
dependency chain runs across chunks), tiny chunks, and one chunk holding a
whole sweep.  In the fused arithmetic both forms fold the same terms with the
same fused operations, so they agree with each other bit for bit too.
"""
import numpy as np
import pytest

import oracle as O
from mojopetsc4py import PETSc, _lib, gallery

pytestmark = pytest.mark.gpu

def _laplacian_box(nx, ny, nz):
    """7-point Laplacian on an nx x ny x nz grid, x fastest (ragged bricks)."""
    n = nx * ny * nz
    p = np.arange(n, dtype=np.int64)
    ix, iy, iz = p % nx, (p // nx) % ny, p // (nx * ny)
    c = np.stack([np.where(iz > 0, p - nx * ny, -1), np.where(iy > 0, p - nx, -1),
                  np.where(ix > 0, p - 1, -1), p, np.where(ix < nx - 1, p + 1, -1),
                  np.where(iy < ny - 1, p + nx, -1), np.where(iz < nz - 1, p + nx * ny, -1)], 1)
    v = np.where(c == p[:, None], 6.0, -1.0)
    keep = c >= 0
    ip = np.zeros(n + 1, np.int32)
    ip[1:] = np.cumsum(keep.sum(1))
    return ip, c[keep].astype(np.int32), v[keep]


MATRICES = {
    "poisson2d_24": lambda: gallery.laplacian_2d(24),
    "poisson3d_10": lambda: gallery.laplacian_3d(10),
    "poisson3d_13x7x6": lambda: _laplacian_box(13, 7, 6),
    "convdiff_9": lambda: gallery.convection_diffusion_3d(9),
}

# (name, tiles, rows per chunk); 0 rows lets the set-up choose
FORMS = [
    ("level-order", False, 0),
    ("chosen", True, 0),
    ("chunks-32", True, 32),
    ("chunks-100", True, 100),   # cuts 24-row lines and 100-row planes
    ("chunks-777", True, 777),
    ("one-chunk", True, 1024),
]

PCS = [
    ("ilu", {}, {}),
    ("ilu", {"setFactorLevels": 1}, {"levels": 1}),
    ("ilu", {"setFactorOrdering": "rcm"}, {"ordering": "rcm"}),
    ("icc", {}, {}),
    ("sor", {}, {}),
    ("sor", {"setSOROmega": 1.2}, {"omega": 1.2}),
    ("sor", {"setSORSymmetric": False}, {"symmetric": False}),
]


@pytest.fixture(autouse=True)
def _restore_form():
    yield
    _lib.set_sweep_form(True, 0)
    _lib.set_sweep_bricks(0, 0, 0, 0)


def _mat(ip, ix, v):
    n = len(ip) - 1
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    return A


def _pc(pt, A, opts):
    pc = PETSc.PC().create()
    pc.setType(pt)
    for k, val in opts.items():
        getattr(pc, k)(val)
    pc.setOperators(A)
    pc.setUp()
    return pc


def _apply(pc, x):
    y = PETSc.Vec().createSeq(len(x))
    pc.apply(PETSc.Vec().createWithArray(np.asarray(x, dtype=np.float64)), y)
    return y.getArray().copy()


@pytest.mark.parametrize("form,tiles,rows", FORMS, ids=[f[0] for f in FORMS])
@pytest.mark.parametrize("pt,gopts,oopts", PCS)
@pytest.mark.parametrize("name", sorted(MATRICES))
def test_sweep_forms_bit_exact(name, pt, gopts, oopts, form, tiles, rows):
    if pt == "icc" and name == "convdiff_9":
        pytest.skip("IC is for symmetric operators")
    ip, ix, v = MATRICES[name]()
    n = len(ip) - 1
    _lib.set_sweep_form(tiles, rows)
    pc = _pc(pt, _mat(ip, ix, v), gopts)
    got = _lib.sweep_form(pc._handle())
    if rows:
        # a forced chunk size is taken whenever the chunk fits in shared memory
        assert got["forward"]["tiled"] and got["backward"]["tiled"], got
        assert got["forward"]["rows_per_chunk"] == min(rows, n)
    elif not tiles:
        assert not got["forward"]["tiled"] and not got["backward"]["tiled"], got
    x = np.random.default_rng(5).normal(size=n)
    want = O.OraclePC(pt, ip, ix, v, **oopts).apply(x)
    np.testing.assert_array_equal(_apply(pc, x), want)
    # a second apply reuses the sweeps' ticket and flag state
    x2 = np.random.default_rng(6).normal(size=n)
    np.testing.assert_array_equal(_apply(pc, x2), O.OraclePC(pt, ip, ix, v, **oopts).apply(x2))


# (name, lines of a brick, CTA cap); 0 lines lets the set-up choose
BRICKS = [
    ("bricks-chosen", 0, 0),
    ("bricks-4", 4, 0),
    ("bricks-1", 1, 0),      # one line a brick: every j - 1 value crosses a brick
    ("bricks-8", 8, 0),
    ("bricks-3", 3, 0),      # cuts 24-, 10-, 9- and 7-line planes unevenly
    ("bricks-planes", 128, 0),  # capped at the grid: one plane a brick
    ("bricks-2-3ctas", 2, 3),   # three CTAs walk every brick in turn
]


@pytest.mark.parametrize("form,bj,ctas", BRICKS, ids=[f[0] for f in BRICKS])
@pytest.mark.parametrize("pt,gopts,oopts", PCS)
@pytest.mark.parametrize("name", sorted(MATRICES))
def test_brick_form_bit_exact(name, pt, gopts, oopts, form, bj, ctas):
    """The brick form wherever the sweep's dependencies are the unit steps of
    the grid (ILU(0), IC(0), SOR in natural order); fill-in (ILU(1)) and a
    reordering (RCM) break that structure and keep the other forms."""
    if pt == "icc" and name == "convdiff_9":
        pytest.skip("IC is for symmetric operators")
    ip, ix, v = MATRICES[name]()
    n = len(ip) - 1
    _lib.set_sweep_bricks(2, bj, 0, ctas)
    pc = _pc(pt, _mat(ip, ix, v), gopts)
    got = _lib.sweep_bricks(pc._handle())
    structured = not ({"setFactorLevels", "setFactorOrdering"} & set(gopts))
    assert got["forward"]["brick"] == structured and got["backward"]["brick"] == structured, got
    if structured and bj:
        nx, ny, _ = got["forward"]["grid"]
        assert got["forward"]["lines"] == (min(bj, nx, ny), 1)
    x = np.random.default_rng(5).normal(size=n)
    want = O.OraclePC(pt, ip, ix, v, **oopts).apply(x)
    np.testing.assert_array_equal(_apply(pc, x), want)
    x2 = np.random.default_rng(6).normal(size=n)
    np.testing.assert_array_equal(_apply(pc, x2), O.OraclePC(pt, ip, ix, v, **oopts).apply(x2))


@pytest.mark.fma
@pytest.mark.parametrize("pt", ["ilu", "icc", "sor"])
def test_fused_forms_agree(pt):
    ip, ix, v = gallery.laplacian_2d(40)
    n = len(ip) - 1
    x = np.random.default_rng(8).normal(size=n)
    out = []
    for tiles, rows, bricks in ((False, 0, 0), (True, 160, 0), (True, 333, 0), (False, 0, 2)):
        _lib.set_sweep_form(tiles, rows)
        _lib.set_sweep_bricks(bricks)
        out.append(_apply(_pc(pt, _mat(ip, ix, v), {}), x))
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])
    np.testing.assert_array_equal(out[0], out[3])
    # and the fused sweeps stay within rounding of the reference's
    want = O.OraclePC(pt, ip, ix, v).apply(x)
    np.testing.assert_allclose(out[0], want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


@pytest.mark.parametrize("tiles,rows,bricks", [(False, 0, 0), (True, 64, 0), (False, 0, 2)])
def test_solves_match_the_oracle_in_every_form(tiles, rows, bricks):
    """A whole captured CG+ICC and GMRES+ILU solve on each form: same
    iteration count and reason as the oracle, iterate to 1e-10."""
    ip, ix, v = gallery.laplacian_2d(32)
    n = len(ip) - 1
    b = np.random.default_rng(5).normal(size=n)
    _lib.set_sweep_form(tiles, rows)
    _lib.set_sweep_bricks(bricks)
    for kt, pt in (("cg", "icc"), ("gmres", "ilu")):
        A = _mat(ip, ix, v)
        pc = PETSc.PC().create()
        pc.setType(pt)
        pc.setOperators(A)
        ksp = PETSc.KSP().create()
        ksp.setPC(pc)
        ksp.setType(kt)
        ksp.setOperators(A)
        ksp.setTolerances(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=2000)
        x = PETSc.Vec().createSeq(n)
        ksp.solve(PETSc.Vec().createWithArray(b), x)
        o = O.solve(kt, ip, ix, v, b, pc_type=pt, rtol=1e-10, atol=1e-50, divtol=1e30,
                    max_it=2000)
        assert ksp.getIterationNumber() == o["its"], (kt, pt)
        assert int(ksp.getConvergedReason()) == o["reason"], (kt, pt)
        xs = x.getArray()
        assert np.linalg.norm(xs - o["x"]) <= 1e-10 * np.linalg.norm(o["x"])


def _sparse_spd(n, density, seed):
    """A random sparse SPD matrix with ragged rows (some rows with no
    off-diagonal entries, some with many)."""
    rng = np.random.default_rng(seed)
    a = np.zeros((n, n))
    for i in range(n):
        k = rng.integers(0, max(1, int(density * n)) + 1)
        cols = rng.choice(n, size=k, replace=False)
        a[i, cols] = rng.uniform(-1, 1, size=k)
    a = a + a.T
    np.fill_diagonal(a, 0.0)
    np.fill_diagonal(a, np.abs(a).sum(axis=1) + 1.0)
    rows, cols = np.nonzero(a)
    ip = np.zeros(n + 1, dtype=np.int64)
    np.add.at(ip, rows + 1, 1)
    return np.cumsum(ip), cols.astype(np.int64), a[rows, cols]


EDGE = {
    "one_row": lambda: (np.array([0, 1]), np.array([0]), np.array([4.0])),
    "two_rows": lambda: (np.array([0, 2, 4]), np.array([0, 1, 0, 1]),
                         np.array([4.0, -1.0, -1.0, 4.0])),
    "diagonal_7": lambda: (np.arange(8), np.arange(7), np.arange(1.0, 8.0)),
    "ragged_60": lambda: _sparse_spd(60, 0.12, 4),
    "wide_rows_40": lambda: _sparse_spd(40, 0.6, 9),   # rows wider than 16: CSR sweeps
}


@pytest.mark.parametrize("form,tiles,rows", [FORMS[0], FORMS[1], FORMS[2], FORMS[3]],
                         ids=[f[0] for f in FORMS[:4]])
@pytest.mark.parametrize("pt", ["ilu", "icc", "sor"])
@pytest.mark.parametrize("name", sorted(EDGE))
def test_sweep_forms_edge_cases(name, pt, form, tiles, rows):
    """Tiny systems, rows without dependencies, ragged and very wide rows:
    every form stays bit-identical to the oracle."""
    ip, ix, v = EDGE[name]()
    n = len(ip) - 1
    _lib.set_sweep_form(tiles, rows)
    pc = _pc(pt, _mat(ip, ix, v), {})
    x = np.random.default_rng(11).normal(size=n)
    np.testing.assert_array_equal(_apply(pc, x), O.OraclePC(pt, ip, ix, v).apply(x))


@pytest.mark.parametrize("pt", ["ilu", "icc", "sor"])
@pytest.mark.parametrize("name", sorted(EDGE))
def test_brick_form_edge_cases(name, pt):
    """The same systems with the brick form allowed wherever the structure is
    found (a two-row line takes it; the others keep the other forms)."""
    ip, ix, v = EDGE[name]()
    n = len(ip) - 1
    _lib.set_sweep_bricks(2, 2, 0, 0)
    pc = _pc(pt, _mat(ip, ix, v), {})
    x = np.random.default_rng(11).normal(size=n)
    np.testing.assert_array_equal(_apply(pc, x), O.OraclePC(pt, ip, ix, v).apply(x))


@pytest.mark.xfail(reason="the reference's IC in a non-natural ordering re-applies row i to "
                          "row r[i] through its diagonal slot label (not an incomplete "
                          "factorization of the permuted matrix); the product computes the "
                          "incomplete Cholesky factor of P A P^T instead",
                   strict=False)
@pytest.mark.parametrize("tiles,rows", [(False, 0), (True, 0), (True, 100)])
@pytest.mark.parametrize("name", ["poisson2d_24", "poisson3d_10"])
def test_icc_in_rcm_order_matches_the_oracle(name, tiles, rows):
    """IC(0) factored in reverse Cuthill-McKee order, applied in every sweep
    form, against the oracle's IC with the same ordering."""
    ip, ix, v = MATRICES[name]()
    n = len(ip) - 1
    _lib.set_sweep_form(tiles, rows)
    pc = _pc("icc", _mat(ip, ix, v), {"setFactorOrdering": "rcm"})
    x = np.random.default_rng(12).normal(size=n)
    want = O.OraclePC("icc", ip, ix, v, ordering="rcm").apply(x)
    np.testing.assert_array_equal(_apply(pc, x), want)


@pytest.mark.parametrize("tiles,rows", [(False, 0), (True, 100)])
def test_icc_in_rcm_order_is_the_incomplete_cholesky_of_the_permuted_matrix(tiles, rows):
    """The device IC(0) in RCM order is the incomplete Cholesky factor of the
    permuted matrix P A P^T (the reference's own result there is not; see the
    expected failure above), to rounding."""
    from helpers import dense_ic0_apply

    ip, ix, v = gallery.laplacian_2d(10)
    n = len(ip) - 1
    A = np.zeros((n, n))
    for i in range(n):
        A[i, ix[ip[i]:ip[i + 1]]] = v[ip[i]:ip[i + 1]]
    _lib.set_sweep_form(tiles, rows)
    pc = _pc("icc", _mat(ip, ix, v), {"setFactorOrdering": "rcm"})
    r = O.OraclePC("icc", ip, ix, v, ordering="rcm")._perms()[0]
    x = np.random.default_rng(12).normal(size=n)
    want = np.empty(n)
    want[r] = dense_ic0_apply(A[np.ix_(r, r)], x[r])
    np.testing.assert_allclose(_apply(pc, x), want, rtol=1e-12, atol=1e-12)
