"""Loads (and if necessary builds) libgpetsc.so, the CUDA library behind the
PETSc classes, and declares its C ABI (include/gpetsc.h) for ctypes.

This replaces the reference's loader (python/mojopetsc4py/_lib.py:107-141),
which compiled and loaded the Mojo library.  The library is built in-tree
with the committed Makefile (nvcc, sm_103a) and loaded from this directory.
There is no CPU fallback: if the library cannot be loaded, or no CUDA device
is present, every device call raises.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "csrc")
LIB = os.environ.get("MOJOPETSC4PY_LIB") or os.path.join(HERE, "libgpetsc.so")

I64 = ctypes.c_int64
I32 = ctypes.c_int32
F64 = ctypes.c_double
P = ctypes.c_void_p
PP = ctypes.POINTER(ctypes.c_void_p)


class BuildError(RuntimeError):
    pass


class GPError(RuntimeError):
    """A gp_* call returned a nonzero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class PcOptions(ctypes.Structure):
    _fields_ = [
        ("type", I32), ("jacobi_type", I32), ("use_abs", I32), ("fix_diag", I32),
        ("rowl1_scale", F64), ("omega", F64), ("fshift", F64), ("sor_flag", I32),
        ("levels", I32), ("ordering", I32), ("reserved", I32),
    ]


class KspOptions(ctypes.Structure):
    _fields_ = [
        ("type", I32), ("normtype", I32), ("pc_side", I32), ("guess_zero", I32),
        ("min_it", I32), ("chknorm", I32), ("convmaxits", I32), ("max_it", I32),
        ("restart", I32), ("orthog", I32), ("cgstype", I32), ("seed_rhs", I32),
        ("rtol", F64), ("atol", F64), ("divtol", F64), ("haptol", F64),
        ("breakdowntol", F64), ("rhs_norm", F64),
    ]


class KspResult(ctypes.Structure):
    _fields_ = [("its", I64), ("reason", I64), ("rnorm", F64)]


# name -> (argtypes, restype) for the gp_* device layer
GP_SIGNATURES = {
    "gp_version": ([], ctypes.c_int),
    "gp_last_error": ([], ctypes.c_char_p),
    "gp_set_arithmetic": ([ctypes.c_int], ctypes.c_int),
    "gp_get_arithmetic": ([], ctypes.c_int),
    "gp_device_count": ([ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "gp_set_device": ([ctypes.c_int], ctypes.c_int),
    "gp_device_alloc": ([PP, I64, P], ctypes.c_int),
    "gp_device_free": ([P, P], ctypes.c_int),
    "gp_host_alloc": ([PP, I64], ctypes.c_int),
    "gp_host_free": ([P], ctypes.c_int),
    "gp_copy": ([P, P, I64, ctypes.c_int, P], ctypes.c_int),
    "gp_stream_synchronize": ([P], ctypes.c_int),
    "gp_coo_assemble": ([I64, I64, I64, P, P, P, P, P, P, P, P, P], ctypes.c_int),
    "gp_dense_to_csr": ([I64, I64, P, I64, P, P, P, P, P], ctypes.c_int),
    "gp_mat_get_csr": ([P, P, P, P, P], ctypes.c_int),
    "gp_mixed_options_default": ([P], None),
    "gp_mixed_create": ([PP], ctypes.c_int),
    "gp_mixed_destroy": ([P], ctypes.c_int),
    "gp_mixed_solve": ([P, P, P, P, P, P, P, P], ctypes.c_int),
    "gp_batch_create": ([PP, I64, P, P, P, P, ctypes.c_int32, P], ctypes.c_int),
    "gp_batch_destroy": ([P], ctypes.c_int),
    "gp_batch_options_default": ([P], None),
    "gp_batch_autotune": ([P, P], ctypes.c_int),
    "gp_batch_tuning": ([P, ctypes.c_int32, P, P, P, P], ctypes.c_int),
    "gp_batch_solve_cg": ([P, P, P, P, P, P, P, P, P], ctypes.c_int),
    "gp_mat_create": ([PP, I64, I64, I64, P, P, P], ctypes.c_int),
    "gp_mat_create_i32": ([PP, I64, I64, I64, P, P, P], ctypes.c_int),
    "gp_mat_destroy": ([P], ctypes.c_int),
    "gp_mat_set_values": ([P, P, ctypes.c_int, P], ctypes.c_int),
    "gp_mat_values_ptr": ([P, PP], ctypes.c_int),
    "gp_mat_info": ([P, P, P, P], ctypes.c_int),
    "gp_mat_spmv_index_bytes": ([P, P], ctypes.c_int),
    "gp_mat_mult": ([P, P, P, P], ctypes.c_int),
    "gp_mat_mult_add": ([P, P, P, P, P], ctypes.c_int),
    "gp_mat_mult_transpose": ([P, P, P, P], ctypes.c_int),
    "gp_mat_transpose": ([P, PP, P], ctypes.c_int),
    "gp_mat_transpose_values": ([P, P, P], ctypes.c_int),
    "gp_mat_outer_on_pattern": ([P, P, P, ctypes.c_double, P, P], ctypes.c_int),
    "gp_mat_get_diagonal": ([P, P, P], ctypes.c_int),
    "gp_vec_map": ([ctypes.c_int, I64, P, P, P, F64, F64, F64, P], ctypes.c_int),
    "gp_vec_maxpy": ([I64, P, I64, P, P, P], ctypes.c_int),
    "gp_vec_reduce": ([ctypes.c_int, I64, P, P, P, P], ctypes.c_int),
    "gp_vec_reduce_static": ([ctypes.c_int, I64, P, P, P, P], ctypes.c_int),
    "gp_vec_minmax": ([I64, P, ctypes.c_int, P, P, P], ctypes.c_int),
    "gp_vec_max_pointwise_divide": ([I64, P, P, P, P], ctypes.c_int),
    "gp_pc_options_default": ([ctypes.POINTER(PcOptions)], None),
    "gp_pc_create": ([PP], ctypes.c_int),
    "gp_pc_destroy": ([P], ctypes.c_int),
    "gp_pc_set_options": ([P, ctypes.POINTER(PcOptions)], ctypes.c_int),
    "gp_pc_setup": ([P, P, P], ctypes.c_int),
    "gp_pc_update_values": ([P, P], ctypes.c_int),
    "gp_wait_probe": ([ctypes.c_int32, ctypes.c_int32, P], ctypes.c_int),
    "gp_set_sweep_form": ([ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "gp_pc_sweep_form": ([P, ctypes.c_int32, P, P, P], ctypes.c_int),
    "gp_set_sweep_bricks": ([ctypes.c_int32] * 4, ctypes.c_int),
    "gp_pc_sweep_bricks": ([P, ctypes.c_int32, P, P], ctypes.c_int),
    "gp_pc_apply": ([P, P, P, P], ctypes.c_int),
    "gp_pc_apply_symmetric": ([P, P, P, P], ctypes.c_int),
    "gp_pc_apply_transpose": ([P, P, P, P], ctypes.c_int),
    "gp_pc_factor_info": ([P, P, P], ctypes.c_int),
    "gp_pc_factor_get": ([P, P, P, P, P, P], ctypes.c_int),
    "gp_ksp_options_default": ([ctypes.POINTER(KspOptions)], None),
    "gp_ksp_create": ([PP], ctypes.c_int),
    "gp_ksp_destroy": ([P], ctypes.c_int),
    "gp_ksp_set_options": ([P, ctypes.POINTER(KspOptions)], ctypes.c_int),
    "gp_ksp_solve": ([P, P, P, P, P, ctypes.POINTER(KspResult), P, I64, P], ctypes.c_int),
    "gp_ksp_stats": ([P, P, P, P], ctypes.c_int),
    "gp_ksp_set_launch_form": ([P, ctypes.c_int], ctypes.c_int),
    "gp_ksp_set_transpose": ([P, ctypes.c_int], ctypes.c_int),
}

_lib = None
_lock = threading.Lock()


def build(force: bool = False, jobs: int = 8) -> str:
    """Compile libgpetsc.so with the Makefile in csrc/ (nvcc, sm_103a)."""
    if force and os.path.exists(LIB):
        os.remove(LIB)
    proc = subprocess.run(["make", "-s", f"-j{jobs}", "-C", CSRC], capture_output=True,
                          text=True)
    if proc.returncode != 0 or not os.path.exists(LIB):
        raise BuildError((proc.stderr or proc.stdout).strip()[-4000:])
    return LIB


def lib() -> ctypes.CDLL:
    """The loaded library, built first when it is missing."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not os.path.exists(LIB):
                    build()
                handle = ctypes.CDLL(LIB)
                for name, (argtypes, restype) in GP_SIGNATURES.items():
                    fn = getattr(handle, name)
                    fn.argtypes = argtypes
                    fn.restype = restype
                _lib = handle
    return _lib


def check(status: int) -> None:
    if status != 0:
        msg = lib().gp_last_error()
        raise GPError(status, msg.decode() if msg else "unknown error")


def device_count() -> int:
    c = ctypes.c_int(0)
    check(lib().gp_device_count(ctypes.byref(c)))
    return c.value


ARITHMETIC = {"exact": 0, "fma": 1, "ordered": 2}


def set_arithmetic(mode: str) -> None:
    """Select the kernels' floating-point form: "exact" (every product and
    sum rounded separately, bit-identical to the reference's loops; parallel
    reductions), "ordered" ("exact" with every reduction summed in the
    reference's blocked order, so whole solves are bit-identical to the
    reference's; slow) or "fma" (fused multiply-adds, the default)."""
    if mode not in ARITHMETIC:
        raise ValueError(f"arithmetic must be one of {sorted(ARITHMETIC)}, got {mode!r}")
    check(lib().gp_set_arithmetic(ARITHMETIC[mode]))


def get_arithmetic() -> str:
    return {v: k for k, v in ARITHMETIC.items()}[lib().gp_get_arithmetic()]


def set_sweep_form(tiles: bool = True, tile_rows: int = 0) -> None:
    """Form of the ILU/IC/SOR triangular sweeps of later PC set-ups:
    `tiles=False` keeps the level-ordered form; `tiles=True` (the default)
    takes the chunked form where its simulated schedule is faster, or with
    `tile_rows` > 0 forces chunks of that many rows.  Both are bit-identical."""
    check(lib().gp_set_sweep_form(1 if tiles else 0, int(tile_rows)))


def set_sweep_bricks(mode: int = 0, lines_j: int = 0, lines_k: int = 0,
                     max_ctas: int = 0) -> None:
    """Brick form of the triangular sweeps of later PC set-ups (grid-structured
    sweeps only): mode 0 never, 1 where modelled faster, 2 whenever the
    structure allows; `lines_j` (1-128) forces the grid lines of a brick, which
    always lies in one plane (`lines_k` 0 or 1); `max_ctas` caps the persistent
    grid.  Bit-identical to the other forms."""
    check(lib().gp_set_sweep_bricks(int(mode), int(lines_j), int(lines_k), int(max_ctas)))


def sweep_bricks(pc_handle) -> dict:
    """Brick form and dims of a set-up PC's forward and backward sweeps."""
    out = {}
    for which, name in ((0, "forward"), (1, "backward")):
        b = ctypes.c_int32()
        d = (ctypes.c_int32 * 5)()
        check(lib().gp_pc_sweep_bricks(pc_handle, which, ctypes.byref(b), d))
        out[name] = {"brick": bool(b.value), "grid": tuple(d[:3]), "lines": tuple(d[3:])}
    return out


def sweep_form(pc_handle, transposed: bool = False) -> dict:
    """The sweep layout a set-up PC got: per sweep, tiled or not, rows per
    chunk and chunk count (with `transposed`, the two sweeps of the transposed
    ILU apply, U^T then L^T)."""
    out = {}
    names = ((2, "first"), (3, "second")) if transposed else ((0, "forward"), (1, "backward"))
    for which, name in names:
        t, r, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        check(lib().gp_pc_sweep_form(pc_handle, which, ctypes.byref(t), ctypes.byref(r),
                                     ctypes.byref(c)))
        out[name] = {"tiled": bool(t.value), "rows_per_chunk": r.value, "chunks": c.value}
    return out


def require_device() -> None:
    """Fail loudly when there is no GPU: there is no CPU path."""
    if device_count() < 1:
        raise RuntimeError(
            "mojopetsc4py (GB300 build) needs a CUDA device; none is visible"
        )
