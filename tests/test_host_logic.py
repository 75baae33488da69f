"""Host-side logic of the PETSc surface that needs no GPU: assembly into CSR,
option setters and their errors, defaults, enums, generators."""
import numpy as np
import pytest

from mojopetsc4py import PETSc, gallery


def test_assembly_setvalues_materialises_sorted_csr():
    A = PETSc.Mat().createSeqAIJ(4, nnz=3)
    A.setValue(2, 3, 1.5)
    A.setValue(2, 0, -1.0)
    A.setValues([0, 1], [1, 0], [1.0, 2.0, 3.0, 4.0])
    A.setValue(2, 3, 0.5, addv=True)
    A.assemble()
    ip, ix, v = A.getValuesCSR()
    assert list(ip) == [0, 2, 4, 6, 6]
    assert list(ix) == [0, 1, 0, 1, 0, 3]
    np.testing.assert_array_equal(v, [2.0, 1.0, 4.0, 3.0, -1.0, 2.0])
    assert A.getValue(2, 3) == 2.0 and A.getValue(3, 3) == 0.0
    assert A.getNNZ() == 6


def test_setvalues_csr_and_transpose_and_from_dense():
    d = np.array([[4.0, -1.0, 0.0], [0.0, 4.0, -2.0], [1.0, 0.0, 3.0]])
    A = PETSc.from_dense(d)
    np.testing.assert_array_equal(A._dense(), d)
    At = A.transpose()
    np.testing.assert_array_equal(At._dense(), d.T)
    assert A.isTranspose(At)
    assert not A.isSymmetric()
    B = A.duplicate(copy=True)
    assert A.equal(B)
    B.scale(2.0)
    np.testing.assert_array_equal(B._dense(), 2 * d)
    C = PETSc.Mat().createSeqAIJ(3)
    C.setValuesCSR(*A.getValuesCSR())
    assert C.equal(A)
    with pytest.raises(ValueError):
        C.setValuesCSR([0, 1], [0], [1.0])


def test_copy_different_pattern_keeps_target_pattern():
    a = PETSc.from_dense(np.array([[1.0, 2.0], [0.0, 3.0]]))
    b = PETSc.from_dense(np.array([[9.0, 0.0], [9.0, 9.0]]))
    a.copy(b, structure=PETSc.Mat.Structure.DIFFERENT_NONZERO_PATTERN)
    np.testing.assert_array_equal(b._dense(), [[1.0, 0.0], [0.0, 3.0]])


def test_ksp_defaults_and_setters():
    k = PETSc.KSP().create()
    assert k.getType() == "gmres"
    assert k.getTolerances() == (1e-5, 1e-50, 1e4, 1000)
    assert k._convmaxits == 0
    k.setTolerances(max_it=5)
    assert k._convmaxits == 1  # reaching max_it then reports CONVERGED_ITS
    with pytest.raises(NotImplementedError):
        k.setType("minres")
    with pytest.raises(TypeError):
        k.setType(3)
    with pytest.raises(RuntimeError):
        k.solve(PETSc.Vec().createSeq(2), PETSc.Vec().createSeq(2))
    assert PETSc.KSP.ConvergedReason.CONVERGED_RTOL == 2
    assert PETSc.KSPConvergedReason.DIVERGED_ITS == -3
    assert PETSc.KSP.NormType.PRECONDITIONED == 2


def test_pc_options_and_errors():
    pc = PETSc.PC().create()
    assert pc.getType() == "none"
    with pytest.raises(NotImplementedError):
        pc.setType("gamg")
    with pytest.raises(NotImplementedError):
        pc.setFactorShift("positive_definite")
    with pytest.raises(ValueError):
        pc.setFactorShift("bogus")
    with pytest.raises(NotImplementedError):
        pc.setFactorPivot(1e-12)
    with pytest.raises(NotImplementedError):
        pc.setFactorOrdering("nd")
    pc.setFactorOrdering("rcm")
    with pytest.raises(RuntimeError):
        pc.setUp()
    assert PETSc.PC.Side.RIGHT == 1 and PETSc.PCSide.SYMMETRIC == 2


def test_vec_host_side():
    v = PETSc.Vec().createSeq(6, bsize=2)
    assert v.getSize() == 6 and v.getBlockSize() == 2
    with pytest.raises(ValueError):
        PETSc.Vec().createSeq(5, bsize=2)
    v.setValues([1, 3], [2.0, 4.0])
    v.setValues([1], [1.0], addv=True)
    np.testing.assert_array_equal(v.getArray(), [0, 3, 0, 4, 0, 0])
    w = v.duplicate([1, 2, 3, 4, 5, 6])
    assert w.getValue(5) == 6.0
    with pytest.raises(ValueError):
        v.setArray([1.0])


def test_generators():
    ip, ix, v = gallery.laplacian_2d(8)
    assert ip[-1] == 5 * 64 - 4 * 8 and np.all(np.diff(ip) > 0)
    ip, ix, v = gallery.laplacian_3d(8)
    assert ip[-1] == 7 * 512 - 6 * 64
    for i in range(512):
        cols = ix[ip[i]:ip[i + 1]]
        assert list(cols) == sorted(cols)
    ip, ix, v = gallery.convection_diffusion_3d(6)
    d = np.zeros((216, 216))
    rows = np.repeat(np.arange(216), np.diff(ip))
    d[rows, ix] = v
    assert not np.allclose(d, d.T)
    assert np.all(np.diag(d) > 0)


def test_sys_version():
    assert PETSc.getVersion() == (3, 25, 5)
    assert "PETSc 3.25.5" in PETSc.getVersionInfo()
