"""The drop-in works without PyTorch.

Vec and Mat keep their device copies in libgpetsc.so's own memory
(gp_device_alloc / gp_host_alloc / gp_copy), so `from mojopetsc4py import
PETSc` and a whole KSP solve run in a process where importing torch fails.
Device blocks still share memory with torch, without a copy, through
__cuda_array_interface__.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mojo-petsc4py_gb300")

BLOCK = "import sys\nsys.modules['torch'] = None  # importing torch now raises\n"


def _run(code):
    env = dict(os.environ, PYTHONPATH=PKG)
    r = subprocess.run([sys.executable, "-c", BLOCK + code], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_package_imports_without_torch():
    out = _run(
        "from mojopetsc4py import PETSc, batch, mixed, gallery, adjoint\n"
        "v = PETSc.Vec().createWithArray([1.0, 2.0, 3.0])\n"
        "v.setValue(1, 5.0)\n"
        "print(v.getArray().tolist())\n"
        "print('torch' in sys.modules and sys.modules['torch'] is not None)\n"
    )
    assert out.split("\n")[:2] == ["[1.0, 5.0, 3.0]", "False"]


@pytest.mark.gpu
def test_solve_without_torch():
    out = _run(
        "import numpy as np\n"
        "from mojopetsc4py import PETSc, gallery\n"
        "ip, ix, v = gallery.laplacian_2d(64)\n"
        "n = len(ip) - 1\n"
        "A = PETSc.Mat().createSeqAIJ((n, n)); A.setValuesCSR(ip, ix, v); A.assemble()\n"
        "ksp = PETSc.KSP().create(); ksp.setOperators(A); ksp.setType('cg')\n"
        "ksp.getPC().setType('icc'); ksp.setTolerances(rtol=1e-10, max_it=1000)\n"
        "b = PETSc.Vec().createWithArray(np.ones(n)); x = PETSc.Vec().createSeq(n)\n"
        "ksp.solve(b, x)\n"
        "r = A.createVecLeft(); A.mult(x, r); r.aypx(-1.0, b)\n"
        "print(ksp.getConvergedReason(), r.norm() / b.norm())\n"
    )
    reason, rel = out.split()
    assert int(reason) > 0 and float(rel) < 1e-9


@pytest.mark.gpu
def test_device_array_round_trip_and_zero_copy_view():
    import torch

    from mojopetsc4py import _device as dev

    a = np.random.default_rng(0).normal(size=(1000, 3))
    d = dev.from_host(a)
    assert d.shape == (1000, 3) and d.nbytes == a.nbytes
    np.testing.assert_array_equal(d.to_host(), a)
    t = torch.as_tensor(d, device="cuda")
    assert t.data_ptr() == d.ptr and t.shape == (1000, 3)
    t.mul_(2.0)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.to_host(), 2.0 * a)
    e = dev.DeviceArray(0)
    assert e.ptr == 0 and e.to_host().shape == (0,)
    assert dev.device_view(t)[0] == d.ptr
    assert dev.device_view(a) is None


@pytest.mark.gpu
def test_pinned_host_arrays_are_recycled_and_zeroed():
    from mojopetsc4py import _device as dev

    n = dev.PINNED_MIN * 4
    a = dev.host_zeros(n)
    assert type(a.base).__name__ == "_PinnedBlock"
    p = a.base.ptr
    a[:] = 7.0
    del a
    b = dev.host_zeros(n)  # the same size class comes back from the cache
    assert b.base.ptr == p and not b.any()
