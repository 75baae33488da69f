"""The differentiable solve (mojopetsc4py.adjoint): gradients of
L = ||u - u_obs||^2 with A(kappa) u = b, A the 2-D advection-diffusion operator
(nonsymmetric), against a dense FP64 reference gradient and central finite
differences, on the 32 x 32 sub-case."""
import numpy as np
import pytest

from mojopetsc4py import gallery

pytestmark = pytest.mark.gpu


def case(k=32, seed=13):
    rng = np.random.default_rng(seed)
    corr = 16.0 * k / 256.0          # the 256^2 field's correlation length, in cells
    kappa = np.exp(gallery.gaussian_random_field(k, rng, corr=corr))
    ip, ix, v = gallery.advection_diffusion_2d(kappa, peclet=2.0)
    kappa_obs = kappa * np.exp(0.1 * gallery.gaussian_random_field(k, rng, corr=corr))
    _, _, v_obs = gallery.advection_diffusion_2d(kappa_obs, peclet=2.0)
    n = k * k
    b = np.ones(n)
    u_obs = np.linalg.solve(dense(ip, ix, v_obs, n), b)
    return ip, ix, v, b, u_obs


def dense(ip, ix, v, n):
    a = np.zeros((n, n))
    for i in range(n):
        a[i, ix[ip[i]:ip[i + 1]]] = v[ip[i]:ip[i + 1]]
    return a


def test_transpose_matrix_on_the_device():
    import torch
    from mojopetsc4py.adjoint import SparseSystem

    ip, ix, v, _, _ = case(k=12)
    n = len(ip) - 1
    sysm = SparseSystem(ip, ix)
    sysm.set_values(torch.tensor(v, device="cuda"))
    g = torch.tensor(np.random.default_rng(1).normal(size=n), device="cuda")
    lam = sysm.solve_transpose(g)
    a = dense(ip, ix, v, n)
    np.testing.assert_allclose(a.T @ lam.cpu().numpy(), g.cpu().numpy(), rtol=0, atol=1e-8)


@pytest.mark.parametrize("kt,pt,rtol,tol,prec", [("gmres", "ilu", 1e-13, 1e-8, "fp64"),
                                                 ("bcgs", "jacobi", 1e-12, 1e-6, "fp64"),
                                                 ("gmres", "ilu", 1e-13, 1e-8, "mixed")])
def test_gradient_matches_the_dense_fp64_gradient(kt, pt, rtol, tol, prec):
    import torch
    from mojopetsc4py.adjoint import SparseSystem, sparse_solve

    ip, ix, v, b, u_obs = case()
    n = len(b)
    sysm = SparseSystem(ip, ix, ksp_type=kt, pc_type=pt, rtol=rtol, precision=prec)
    vals = torch.tensor(v, device="cuda", requires_grad=True)
    bt = torch.tensor(b, device="cuda", requires_grad=True)
    uo = torch.tensor(u_obs, device="cuda")
    u = sparse_solve(vals, bt, sysm)
    loss = ((u - uo) ** 2).sum()
    loss.backward()

    a = dense(ip, ix, v, n)
    ud = np.linalg.solve(a, b)
    lam = np.linalg.solve(a.T, 2 * (ud - u_obs))
    rows = np.repeat(np.arange(n), np.diff(ip))
    gv_ref = -lam[rows] * ud[ix]
    uu = u.detach().cpu().numpy()
    assert np.linalg.norm(uu - ud) <= tol * np.linalg.norm(ud)
    gv = vals.grad.cpu().numpy()
    gb = bt.grad.cpu().numpy()
    assert np.linalg.norm(gv - gv_ref) <= tol * np.linalg.norm(gv_ref)
    assert np.linalg.norm(gb - lam) <= tol * np.linalg.norm(lam)


def test_gradient_matches_central_finite_differences():
    import torch
    from mojopetsc4py.adjoint import SparseSystem, sparse_solve

    ip, ix, v, b, u_obs = case()
    sysm = SparseSystem(ip, ix, rtol=1e-14)
    uo = torch.tensor(u_obs, device="cuda")
    bt = torch.tensor(b, device="cuda", requires_grad=True)

    def loss_of(vals_np, b_t):
        vt = torch.tensor(vals_np, device="cuda")
        with torch.no_grad():
            u = sparse_solve(vt, b_t, sysm)
        return float(((u - uo) ** 2).sum())

    vals = torch.tensor(v, device="cuda", requires_grad=True)
    u = sparse_solve(vals, bt, sysm)
    ((u - uo) ** 2).sum().backward()
    gv = vals.grad.cpu().numpy()
    gb = bt.grad.cpu().numpy()

    rng = np.random.default_rng(3)
    for k in rng.choice(len(v), size=6, replace=False):
        h = 1e-5 * abs(v[k])
        vp, vm = v.copy(), v.copy()
        vp[k] += h
        vm[k] -= h
        fd = (loss_of(vp, bt.detach()) - loss_of(vm, bt.detach())) / (2 * h)
        assert abs(fd - gv[k]) <= 1e-4 * abs(gv[k]) + 1e-9, (k, fd, gv[k])
    for i in rng.choice(len(b), size=4, replace=False):
        h = 1e-5
        bp, bm = b.copy(), b.copy()
        bp[i] += h
        bm[i] -= h
        fd = (loss_of(v, torch.tensor(bp, device="cuda"))
              - loss_of(v, torch.tensor(bm, device="cuda"))) / (2 * h)
        assert abs(fd - gb[i]) <= 1e-4 * abs(gb[i]) + 1e-9, (i, fd, gb[i])


def test_mixed_precision_solves_follow_value_changes():
    """The mixed form keeps its FP32 values, factor and captured pass at fixed
    addresses: after every value change both the forward and the adjoint
    solve must meet rtol on the true FP64 residual of the new matrix."""
    import torch
    from mojopetsc4py.adjoint import SparseSystem

    ip, ix, v, b, _ = case(k=24)
    n = len(b)
    sysm = SparseSystem(ip, ix, rtol=1e-11, precision="mixed")
    bt = torch.tensor(b, device="cuda")
    g = torch.tensor(np.random.default_rng(2).normal(size=n), device="cuda")
    for scale in (1.0, 1.7, 0.6):
        vs = v * scale * (1.0 + 0.05 * np.sin(np.arange(len(v))))
        sysm.set_values(torch.tensor(vs, device="cuda"))
        a = dense(ip, ix, vs, n)
        u = sysm.solve(bt).cpu().numpy()
        assert np.linalg.norm(a @ u - b) <= 1e-11 * np.linalg.norm(b) * 1.01
        lam = sysm.solve_transpose(g).cpu().numpy()
        gh = g.cpu().numpy()
        assert np.linalg.norm(a.T @ lam - gh) <= 1e-11 * np.linalg.norm(gh) * 1.01
        assert sysm.forward_solver.passes >= 1 and sysm.adjoint_solver.passes >= 1
