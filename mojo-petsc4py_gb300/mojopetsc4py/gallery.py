"""Seeded test matrices for the Krylov path, as int32/float64 CSR triples.

These are the workloads the solver is measured and checked on: the 2-D
5-point and 3-D 7-point Poisson operators, a nonsymmetric upwind
convection-diffusion operator, random-geometric-graph Laplacians and a 2-D
advection-diffusion operator with a log-normal coefficient.  Every generator
returns `(indptr, indices, values)` with ascending columns in each row, which
is the SeqAIJ layout `Mat.setValuesCSR` takes.
"""

from __future__ import annotations

import numpy as np


def _csr_from_candidates(cands: np.ndarray, vals: np.ndarray):
    """(n, k) candidate columns (-1 = absent, ascending per row) -> CSR."""
    keep = cands >= 0
    counts = keep.sum(axis=1).astype(np.int64)
    indptr = np.zeros(cands.shape[0] + 1, dtype=np.int32)
    indptr[1:] = np.cumsum(counts)
    return indptr, cands[keep].astype(np.int32), vals[keep].astype(np.float64)


def laplacian_2d(k: int):
    """5-point Laplacian on a k x k grid, row-major numbering, 4 on the
    diagonal and -1 off it, Dirichlet boundary folded in.  Same row and column
    order as the reference benchmark's generator (bench/bench.py:64-93)."""
    n = k * k
    p = np.arange(n, dtype=np.int64)
    cands = np.stack([
        np.where(p >= k, p - k, -1),
        np.where(p % k > 0, p - 1, -1),
        p,
        np.where(p % k < k - 1, p + 1, -1),
        np.where(p < n - k, p + k, -1),
    ], axis=1)
    vals = np.where(cands == p[:, None], 4.0, -1.0)
    return _csr_from_candidates(cands, vals)


def laplacian_3d(k: int):
    """7-point Laplacian on a k^3 grid, lexicographic numbering with x fastest,
    6 on the diagonal and -1 off it, off-grid neighbours dropped."""
    n = k * k * k
    p = np.arange(n, dtype=np.int64)
    ix = p % k
    iy = (p // k) % k
    iz = p // (k * k)
    kk = k * k
    cands = np.stack([
        np.where(iz > 0, p - kk, -1),
        np.where(iy > 0, p - k, -1),
        np.where(ix > 0, p - 1, -1),
        p,
        np.where(ix < k - 1, p + 1, -1),
        np.where(iy < k - 1, p + k, -1),
        np.where(iz < k - 1, p + kk, -1),
    ], axis=1)
    vals = np.where(cands == p[:, None], 6.0, -1.0)
    return _csr_from_candidates(cands, vals)


def convection_diffusion_3d(k: int, velocity=(1.0, 0.5, 0.25), peclet: float = 10.0):
    """First-order upwind convection-diffusion on a k^3 grid, scaled by h^2.

    h = 1/(k+1); nu = h max|v| / peclet (cell Peclet number `peclet`).  Row of
    cell c: diagonal 6 nu + h sum(v_i); neighbour c - e_i gets -nu - h v_i
    (upwind, v_i > 0); neighbour c + e_i gets -nu.  Nonsymmetric."""
    n = k * k * k
    h = 1.0 / (k + 1)
    v = np.asarray(velocity, dtype=np.float64)
    nu = h * float(np.max(np.abs(v))) / peclet
    p = np.arange(n, dtype=np.int64)
    ix = p % k
    iy = (p // k) % k
    iz = p // (k * k)
    kk = k * k
    lo = lambda i: -nu - h * v[i]  # noqa: E731
    hi = -nu
    cands = np.stack([
        np.where(iz > 0, p - kk, -1),
        np.where(iy > 0, p - k, -1),
        np.where(ix > 0, p - 1, -1),
        p,
        np.where(ix < k - 1, p + 1, -1),
        np.where(iy < k - 1, p + k, -1),
        np.where(iz < k - 1, p + kk, -1),
    ], axis=1)
    diag = 6.0 * nu + h * float(v.sum())
    vals = np.stack([
        np.full(n, lo(2)), np.full(n, lo(1)), np.full(n, lo(0)), np.full(n, diag),
        np.full(n, hi), np.full(n, hi), np.full(n, hi),
    ], axis=1)
    return _csr_from_candidates(cands, vals)


def rgg_laplacian(n: int, rng: np.random.Generator, mean_degree: float = 8.0,
                  shift: float = 1e-2):
    """Random geometric graph Laplacian L = D - W + shift*I on n points in the
    unit square, radius sqrt(mean_degree/(pi n)), edge weights U[0.5, 2]."""
    from scipy.spatial import cKDTree

    pts = rng.random((n, 2))
    radius = np.sqrt(mean_degree / (np.pi * n))
    pairs = cKDTree(pts).query_pairs(radius, output_type="ndarray")
    w = rng.uniform(0.5, 2.0, size=len(pairs))
    i = np.concatenate([pairs[:, 0], pairs[:, 1], np.arange(n)])
    j = np.concatenate([pairs[:, 1], pairs[:, 0], np.arange(n)])
    deg = np.zeros(n)
    np.add.at(deg, pairs[:, 0], w)
    np.add.at(deg, pairs[:, 1], w)
    v = np.concatenate([-w, -w, deg + shift])
    order = np.lexsort((j, i))
    i, j, v = i[order], j[order], v[order]
    indptr = np.zeros(n + 1, dtype=np.int32)
    np.add.at(indptr, i + 1, 1)
    indptr = np.cumsum(indptr).astype(np.int32)
    return indptr, j.astype(np.int32), v.astype(np.float64)


def hub_laplacian(n: int, hubs: int, spokes: int, seed: int = 9, shift: float = 1e-2):
    """A graph Laplacian with a few very long rows: the path 0-1-...-(n-1)
    with unit weights plus `hubs` rows each joined to `spokes` distinct random
    rows (weights U[0.5, 2]); L = D - W + shift*I (SPD).  Row lengths are 2-3
    except the hubs' (~spokes), the skew a one-thread-a-row SpMV handles worst."""
    rng = np.random.default_rng(seed)
    pi = np.arange(n - 1)
    ei, ej, ew = [pi], [pi + 1], [np.ones(n - 1)]
    for h in range(hubs):
        js = rng.choice(np.arange(h + 2, n), size=spokes, replace=False)
        ei.append(np.full(spokes, h))
        ej.append(js)
        ew.append(rng.uniform(0.5, 2.0, size=spokes))
    ei, ej, ew = np.concatenate(ei), np.concatenate(ej), np.concatenate(ew)
    # an edge drawn twice (two hubs' spokes meeting) keeps the sum of its weights
    key = np.minimum(ei, ej).astype(np.int64) * n + np.maximum(ei, ej)
    key, inv = np.unique(key, return_inverse=True)
    w = np.zeros(len(key))
    np.add.at(w, inv, ew)
    a, b = key // n, key % n
    deg = np.zeros(n)
    np.add.at(deg, a, w)
    np.add.at(deg, b, w)
    i = np.concatenate([a, b, np.arange(n)])
    j = np.concatenate([b, a, np.arange(n)])
    v = np.concatenate([-w, -w, deg + shift])
    order = np.lexsort((j, i))
    i, j, v = i[order], j[order], v[order]
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(indptr, i + 1, 1)
    indptr = np.cumsum(indptr).astype(np.int32)
    return indptr, j.astype(np.int32), v.astype(np.float64)


def rgg_batch(count: int = 512, seed: int = 11, nmin: int = 1024, nmax: int = 65536):
    """`count` RGG Laplacians with sizes log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=count))).astype(int)
    return [rgg_laplacian(int(s), rng) for s in sizes]


def gaussian_random_field(k: int, rng: np.random.Generator, corr: float = 16.0):
    """Unit-variance field on a k x k grid: white noise filtered in Fourier
    space with a Gaussian kernel of length `corr` cells."""
    noise = rng.normal(size=(k, k))
    fx = np.fft.fftfreq(k)
    kx, ky = np.meshgrid(fx, fx, indexing="ij")
    filt = np.exp(-0.5 * (2 * np.pi * corr) ** 2 * (kx ** 2 + ky ** 2))
    field = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    field -= field.mean()
    return field / field.std()


def advection_diffusion_2d(kappa: np.ndarray, peclet: float = 2.0,
                           velocity=(1.0, 0.0)):
    """Steady advection-diffusion on a k x k grid with cell coefficient
    `kappa` (face value = arithmetic mean of the two cells), constant velocity
    scaled to a mesh Peclet number |v| h / mean(kappa) = `peclet`, first-order
    upwind, Dirichlet boundary, rows scaled by h^2.  Nonsymmetric."""
    k = kappa.shape[0]
    n = k * k
    h = 1.0 / (k + 1)
    vdir = np.asarray(velocity, dtype=np.float64)
    vmag = peclet * float(kappa.mean()) / h
    v = vdir / np.linalg.norm(vdir) * vmag
    p = np.arange(n, dtype=np.int64)
    ix = p % k
    iy = p // k
    kap = kappa.reshape(-1)

    def face(q, ok):
        return np.where(ok, 0.5 * (kap + kap[np.where(ok, q, p)]), kap)

    kxm = face(p - 1, ix > 0)
    kxp = face(p + 1, ix < k - 1)
    kym = face(p - k, iy > 0)
    kyp = face(p + k, iy < k - 1)
    # upwind convection scaled by h (the operator is multiplied through by h^2)
    cxm = h * max(v[0], 0.0)
    cxp = h * max(-v[0], 0.0)
    cym = h * max(v[1], 0.0)
    cyp = h * max(-v[1], 0.0)
    diag = kxm + kxp + kym + kyp + cxm + cxp + cym + cyp
    cands = np.stack([
        np.where(iy > 0, p - k, -1),
        np.where(ix > 0, p - 1, -1),
        p,
        np.where(ix < k - 1, p + 1, -1),
        np.where(iy < k - 1, p + k, -1),
    ], axis=1)
    vals = np.stack([-kym - cym, -kxm - cxm, diag, -kxp - cxp, -kyp - cyp], axis=1)
    return _csr_from_candidates(cands, vals)


def tridiag(n: int, diag: float = 4.0, off: float = -1.0):
    """Tridiagonal CSR (the reference's README example matrix)."""
    rows = []
    cols = []
    vals = []
    indptr = [0]
    for i in range(n):
        for j in sorted({max(i - 1, 0), i, min(i + 1, n - 1)}):
            cols.append(j)
            vals.append(diag if j == i else off)
        indptr.append(len(cols))
        rows.append(i)
    return (np.array(indptr, dtype=np.int32), np.array(cols, dtype=np.int32),
            np.array(vals, dtype=np.float64))
