"""Shared builders for the tests: CSR generators, dense helpers, oracle calls."""
import numpy as np

import oracle as O
from mojopetsc4py import gallery


def tridiag_dense(n, d=4.0, off=-1.0):
    a = np.zeros((n, n))
    for i in range(n):
        a[i, i] = d
        if i:
            a[i, i - 1] = off
        if i + 1 < n:
            a[i, i + 1] = off
    return a


def dense_to_csr(a):
    rows, cols = np.nonzero(a)
    indptr = np.zeros(a.shape[0] + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    return np.cumsum(indptr), cols.astype(np.int64), a[rows, cols].astype(np.float64)


def spd_dense(n, seed=0):
    rng = np.random.default_rng(seed)
    m = rng.normal(size=(n, n))
    return m + m.T + 2 * n * np.eye(n)


def nonsym_banded(n, seed=0, bw=3):
    """A diagonally dominant nonsymmetric banded matrix."""
    rng = np.random.default_rng(seed)
    a = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - bw), min(n, i + bw + 1)):
            a[i, j] = rng.uniform(-1, 1)
        a[i, i] = 2 * bw + 2.0
    return a


def lap2d(k):
    return gallery.laplacian_2d(k)


def oracle_solve(kt, ip, ix, v, b, pt="none", **kw):
    return O.solve(kt, ip, ix, v, b, pc_type=pt, **kw)


def dense_ic0_apply(B, x):
    """IC(0) of B on B's lower pattern, L L^T, applied to x (dense, small)."""
    m = B.shape[0]
    L = np.tril(B).copy()
    pat = np.tril(B) != 0
    for k in range(m):
        L[k, k] = np.sqrt(L[k, k])
        for i in range(k + 1, m):
            if pat[i, k]:
                L[i, k] /= L[k, k]
        for j in range(k + 1, m):
            for i in range(j, m):
                if pat[i, j] and pat[i, k] and pat[j, k]:
                    L[i, j] -= L[i, k] * L[j, k]
    return np.linalg.solve(L @ L.T, x)
