"""The CPU oracle against the reference's published known answers and numpy
closed forms (no GPU).  These pin the checker before it checks the GPU."""
import json
import os

import numpy as np
import pytest

import oracle as O
from helpers import dense_to_csr, lap2d, oracle_solve, spd_dense, tridiag_dense

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "published.json")))


def a(x):
    return x.ctypes.data


CASES = [(key, int(k), its) for key, d in GOLD["iterations"].items() for k, its in d.items()
         if int(k) <= 64 or key in ("cg+none", "cg+ilu", "cg+icc")]


@pytest.mark.parametrize("key,k,want", CASES)
def test_published_iteration_counts(key, k, want):
    kt, pt = key.split("+")
    ip, ix, v = lap2d(k)
    b = np.random.default_rng(5).normal(size=k * k)
    r = oracle_solve(kt, ip, ix, v, b, pt, rtol=1e-10, atol=1e-50, divtol=1e30, max_it=2000)
    if kt == "bcgs":
        assert abs(r["its"] - want) <= GOLD["bcgs_tolerance"]
    else:
        assert r["its"] == want
    assert r["reason"] in (2, 4)


def test_readme_example():
    ex = GOLD["readme_example"]
    ip, ix, v = dense_to_csr(tridiag_dense(ex["n"]))
    r = oracle_solve("cg", ip, ix, v, np.ones(ex["n"]), "ilu", rtol=ex["rtol"],
                     max_it=ex["max_it"])
    assert r["its"] == ex["its"]
    res = np.ones(ex["n"]) - tridiag_dense(ex["n"]) @ r["x"]
    # same magnitude as the published round-off (the last bits depend on the
    # CPU's SIMD width and contraction)
    assert np.linalg.norm(res) < 1e-14


def test_vec_kernels_against_numpy():
    L = O.lib()
    rng = np.random.default_rng(0)
    for n in (0, 1, 3, 4, 15, 16, 17, 63, 64, 65, 16383, 16384, 16385):
        x, y = rng.normal(size=n), rng.normal(size=n)
        out = np.zeros(2)
        L.mp_vec_dot(a(x), a(y), a(out), n)
        assert out[0] == pytest.approx(float(x @ y), rel=1e-12, abs=1e-12)
        L.mp_vec_norm(a(x), 1, a(out), n)
        assert out[0] == pytest.approx(float(np.linalg.norm(x)), rel=1e-12, abs=1e-300)
        L.mp_vec_norm(a(x), 4, a(out), n)
        assert out[0] == pytest.approx(float(np.abs(x).sum()), rel=1e-12, abs=1e-300)
        assert out[1] == pytest.approx(float(np.linalg.norm(x)), rel=1e-12, abs=1e-300)
        L.mp_vec_sum(a(x), a(out), n)
        assert out[0] == pytest.approx(float(x.sum()), rel=1e-10, abs=1e-10)
        s, r = np.zeros(1), np.zeros(1)
        L.mp_vec_dot_norm2(a(x), a(y), a(s), a(r), n)
        assert s[0] == pytest.approx(float(x @ y), rel=1e-12, abs=1e-12)
        assert r[0] == pytest.approx(float(x @ x), rel=1e-12, abs=1e-300)
    n = 37
    x, y, z = rng.normal(size=n), rng.normal(size=n), rng.normal(size=n)
    w = y.copy()
    L.mp_vec_axpy(a(w), 2.5, a(x), n)
    np.testing.assert_array_equal(w, y + 2.5 * x)
    w = y.copy()
    L.mp_vec_aypx(a(w), -1.5, a(x), n)
    np.testing.assert_array_equal(w, x + -1.5 * y)
    w = z.copy()
    L.mp_vec_axpbypcz(a(w), 1.5, -2.0, 0.5, a(x), a(y), n)
    np.testing.assert_array_equal(w, 1.5 * x + -2.0 * y + 0.5 * z)
    w = np.zeros(n)
    L.mp_vec_waxpy(a(w), -0.25, a(x), a(y), n)
    np.testing.assert_array_equal(w, -0.25 * x + y)
    idx, val = np.zeros(1, dtype=np.int64), np.zeros(1)
    xx = np.array([1.0, 5.0, -2.0, 5.0, 0.0])
    L.mp_vec_max(a(xx), a(idx), a(val), 5)
    assert (idx[0], val[0]) == (1, 5.0)
    L.mp_vec_min(a(xx), a(idx), a(val), 5)
    assert (idx[0], val[0]) == (2, -2.0)
    r0 = np.array([0.0, 2.0, -4.0, 1e-20])
    L.mp_vec_reciprocal(a(r0), 4)
    np.testing.assert_array_equal(r0, [0.0, 0.5, -0.25, 1e20])


def test_mat_kernels_against_numpy():
    L = O.lib()
    dense = spd_dense(12, 3)
    dense[np.abs(dense) < 1.0] = 0.0
    ip, ix, v = dense_to_csr(dense)
    x = np.random.default_rng(2).normal(size=12)
    y = np.zeros(12)
    L.mp_mat_mult(a(x), a(y), a(ip), a(ix), a(v), 12)
    np.testing.assert_allclose(y, dense @ x, rtol=1e-13, atol=1e-13)
    yt = np.full(12, 9.0)
    L.mp_mat_mult_transpose(a(x), a(yt), a(ip), a(ix), a(v), 12, 12)
    np.testing.assert_allclose(yt, dense.T @ x, rtol=1e-13, atol=1e-13)
    ya = np.ones(12)
    L.mp_mat_mult_add(a(x), a(ya), a(ip), a(ix), a(v), 12)
    np.testing.assert_allclose(ya, dense @ x + 1.0, rtol=1e-13, atol=1e-13)


def test_sor_matches_numpy_symmetric_sweep():
    dense = tridiag_dense(9)
    ip, ix, v = dense_to_csr(dense)
    x = np.random.default_rng(51).normal(size=9)
    for omega, fshift in ((1.0, 0.0), (1.3, 0.25)):
        pc = O.OraclePC("sor", ip, ix, v, omega=omega, fshift=fshift)
        y = pc.apply(x)
        d = np.diag(dense)
        idiag = 1.0 / d if (omega == 1.0 and fshift <= 0) else omega / (fshift + d)
        want, t = np.zeros(9), np.zeros(9)
        for i in range(9):
            t[i] = x[i] - dense[i, :i] @ want[:i]
            want[i] = t[i] * idiag[i]
        for i in range(8, -1, -1):
            s = t[i] - dense[i, i + 1:] @ want[i + 1:]
            want[i] = (1 - omega) * want[i] + s * idiag[i]
        np.testing.assert_allclose(y, want, rtol=0, atol=1e-13)


@pytest.mark.parametrize("kind", ["ilu", "icc"])
def test_incomplete_factors_exact_on_tridiagonal(kind):
    dense = tridiag_dense(15)
    ip, ix, v = dense_to_csr(dense)
    b = np.random.default_rng(54).normal(size=15)
    pc = O.OraclePC(kind, ip, ix, v)
    np.testing.assert_allclose(pc.apply(b), np.linalg.solve(dense, b), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("kt", ["cg", "gmres", "fgmres", "bcgs"])
def test_solutions_against_dense_solve(kt):
    dense = tridiag_dense(30)
    ip, ix, v = dense_to_csr(dense)
    b = np.random.default_rng(56).normal(size=30)
    r = oracle_solve(kt, ip, ix, v, b, "jacobi", rtol=1e-12, max_it=200, restart=20)
    np.testing.assert_allclose(r["x"], np.linalg.solve(dense, b), rtol=1e-8, atol=1e-8)
    assert r["reason"] in (2, 3)


def test_ilu_levels_factor_layout():
    """Level-of-fill ILU(1) layout invariants (the reference's test_factor_layout)."""
    ip, ix, v = lap2d(6)
    pc = O.OraclePC("ilu", ip, ix, v, levels=1)
    f = pc.factor
    n = 36
    for i in range(n):
        assert f["bj"][f["bdiag"][i]] == i
        lower = f["bj"][f["bi"][i]:f["bi"][i + 1]]
        assert all(c < i for c in lower) and list(lower) == sorted(lower)
        upper = f["bj"][f["bdiag"][i + 1] + 1:f["bdiag"][i]]
        assert all(c > i for c in upper) and list(upper) == sorted(upper)
