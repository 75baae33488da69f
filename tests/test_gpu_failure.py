"""Failure detection without a GPU fault: the sweeps' device wait runs out
of its budget on a flag that nothing sets, the kernel records GP_ERR_TIMEOUT
and returns, the host reads the status, and the context stays usable."""
import numpy as np
import pytest

from mojopetsc4py import PETSc, _lib, gallery

pytestmark = pytest.mark.gpu

GP_ERR_TIMEOUT = 3


def test_wait_on_a_flag_nothing_sets_times_out_with_a_status():
    lib = _lib.lib()
    st = lib.gp_wait_probe(2000, 0, None)
    assert st == GP_ERR_TIMEOUT
    assert b"budget" in lib.gp_last_error()


def test_wait_on_a_ready_flag_returns_at_once():
    assert _lib.lib().gp_wait_probe(2000, 1, None) == 0


def test_the_context_stays_usable_after_a_timeout():
    lib = _lib.lib()
    assert lib.gp_wait_probe(500, 0, None) == GP_ERR_TIMEOUT
    ip, ix, v = gallery.laplacian_2d(16)
    n = 256
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    ksp = PETSc.KSP().create()
    ksp.setOperators(A)
    ksp.setType("cg")
    ksp.getPC().setType("ilu")
    ksp.setTolerances(rtol=1e-10)
    b = PETSc.Vec().createWithArray(np.ones(n))
    x = PETSc.Vec().createSeq(n)
    ksp.solve(b, x)
    assert ksp.getConvergedReason() > 0
    assert lib.gp_wait_probe(500, 1, None) == 0
