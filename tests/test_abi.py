"""The C ABI: libgpetsc.so loads and exports every entry point include/gpetsc.h
declares, including the reference's 59 mp_* names (src/capi.mojo); the
oracle exports the same 59 (no GPU needed: nothing here computes)."""
import ctypes
import os
import re

import oracle as O
from mojopetsc4py import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpetsc.h")

# the reference's exported set, src/capi.mojo:32-424 (tests/test_exported_kernels.py:1100-1134)
REFERENCE_EXPORTS = {
    "mp_mat_mult", "mp_mat_mult_add", "mp_mat_mult_transpose", "mp_mat_get_diagonal",
    "mp_mat_scale", "mp_mat_zero_entries", "mp_mat_get_diagonal_markers",
    "mp_vec_pointwise_mult", "mp_vec_pointwise_divide", "mp_vec_pointwise_min",
    "mp_vec_pointwise_max", "mp_vec_pointwise_max_abs", "mp_vec_norm", "mp_vec_dot",
    "mp_vec_tdot", "mp_vec_dot_norm2", "mp_vec_sum", "mp_vec_mean", "mp_vec_max",
    "mp_vec_min", "mp_vec_normalize", "mp_vec_reciprocal", "mp_vec_exp", "mp_vec_log",
    "mp_vec_sqrtabs", "mp_vec_chop", "mp_vec_abs", "mp_vec_conjugate", "mp_vec_copy",
    "mp_vec_swap", "mp_vec_set", "mp_vec_zero_entries", "mp_vec_scale", "mp_vec_shift",
    "mp_vec_axpy", "mp_vec_aypx", "mp_vec_axpby", "mp_vec_axpbypcz", "mp_vec_waxpy",
    "mp_vec_maxpy", "mp_vec_max_pointwise_divide", "mp_pc_jacobi_setup",
    "mp_pc_jacobi_setup_symmetric", "mp_pc_jacobi_apply", "mp_pc_sor_apply", "mp_pc_ilu_apply",
    "mp_pc_icc_apply", "mp_pc_ilu_numeric", "mp_pc_icc_numeric", "mp_ilu_symbolic_ilu0",
    "mp_ilu_symbolic", "mp_ilu_contiguous_lu", "mp_icc_symbolic", "mp_icc_contiguous_cholesky",
    "mp_ordering_rcm", "mp_ksp_solve_cg", "mp_ksp_solve_bcgs", "mp_ksp_solve_gmres",
    "mp_ksp_solve_fgmres",
}


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b((?:gp|mp)_[a-z0-9_]+)\s*\(", text))


def test_reference_export_count():
    assert len(REFERENCE_EXPORTS) == 59


def test_header_declares_the_reference_abi():
    assert REFERENCE_EXPORTS <= declared()


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB)
    missing = sorted(n for n in declared() if not hasattr(lib, n))
    assert not missing, missing


def test_python_signature_table_matches_header():
    assert set(_lib.GP_SIGNATURES) <= declared()
    gp_declared = {n for n in declared() if n.startswith("gp_")}
    assert gp_declared - set(_lib.GP_SIGNATURES) <= {"gp_pc_options_default", "gp_ksp_options_default"} | set()


def test_oracle_exports_the_same_59():
    lib = O.lib()
    assert all(hasattr(lib, n) for n in REFERENCE_EXPORTS)
    assert set(O.SIGNATURES) == REFERENCE_EXPORTS


def test_loads_without_a_device():
    """Version and device count answer on a host without a GPU."""
    lib = _lib.lib()
    assert lib.gp_version() >= 100
    assert _lib.device_count() >= 0


def test_brick_settings_are_checked_on_the_host():
    """The brick form's lines lie in one plane: lines_k above 1, or more than
    128 lines, is an argument error (no device needed)."""
    lib = _lib.lib()
    assert lib.gp_set_sweep_bricks(0, 0, 2, 0) == 1
    assert lib.gp_set_sweep_bricks(0, 129, 1, 0) == 1
    assert lib.gp_set_sweep_bricks(0, 64, 1, 0) == 0
    assert lib.gp_set_sweep_bricks(0, 0, 0, 0) == 0
