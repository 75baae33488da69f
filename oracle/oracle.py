"""ctypes binding and host-side driver for the CPU oracle.

TEST INFRASTRUCTURE ONLY.  Only `tests/`, `__graft_entry__.smoke()` and the
`cpu_baseline` / reference leg of `bench.py` import this module, and only as
the checker or as the timed CPU restatement of the reference; the product
package never imports it.

`liboracle.so` exports the reference's host C ABI (src/capi.mojo).  This
module adds the host logic that the reference keeps in Python around that ABI
-- the PC set-up with its retry-on-negative symbolic protocol
(python/mojopetsc4py/PETSc/PC.py:315-492), the cfg/cfgi/pci block packing
(KSP.py:457-494, PC.py:495-547) and the solve dispatch (KSP.py:367-449) -- so
a test can run the reference's whole CPU path on the same inputs as the GPU.
"""

from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# the timing build of the CPU baseline (FMA contraction; see the Makefile)
LIB_TIMING = os.path.join(HERE, "_build", "liboracle_timing.so")

I = ctypes.c_int64
F = ctypes.c_double
P = ctypes.c_void_p

# name -> (argtypes, restype); the reference's _lib.py:23-87 table with
# addresses typed as pointers
SIGNATURES = {
    "mp_mat_mult": ([P, P, P, P, P, I], None),
    "mp_mat_mult_add": ([P, P, P, P, P, I], None),
    "mp_mat_mult_transpose": ([P, P, P, P, P, I, I], None),
    "mp_mat_get_diagonal": ([P, P, P, P, I], None),
    "mp_mat_scale": ([P, I, F], None),
    "mp_mat_zero_entries": ([P, I], None),
    "mp_vec_pointwise_mult": ([P, P, P, I], None),
    "mp_vec_pointwise_divide": ([P, P, P, I], None),
    "mp_vec_pointwise_min": ([P, P, P, I], None),
    "mp_vec_pointwise_max": ([P, P, P, I], None),
    "mp_vec_pointwise_max_abs": ([P, P, P, I], None),
    "mp_vec_norm": ([P, I, P, I], None),
    "mp_vec_dot": ([P, P, P, I], None),
    "mp_vec_tdot": ([P, P, P, I], None),
    "mp_vec_sum": ([P, P, I], None),
    "mp_vec_mean": ([P, P, I], None),
    "mp_vec_dot_norm2": ([P, P, P, P, I], None),
    "mp_vec_max": ([P, P, P, I], None),
    "mp_vec_min": ([P, P, P, I], None),
    "mp_vec_normalize": ([P, P, I], None),
    "mp_vec_reciprocal": ([P, I], None),
    "mp_vec_exp": ([P, I], None),
    "mp_vec_log": ([P, I], None),
    "mp_vec_sqrtabs": ([P, I], None),
    "mp_vec_chop": ([P, I, F], None),
    "mp_vec_abs": ([P, I], None),
    "mp_vec_conjugate": ([P, I], None),
    "mp_vec_copy": ([P, P, I], None),
    "mp_vec_swap": ([P, P, I], None),
    "mp_vec_set": ([P, F, I], None),
    "mp_vec_zero_entries": ([P, I], None),
    "mp_vec_scale": ([P, F, I], None),
    "mp_vec_shift": ([P, F, I], None),
    "mp_vec_axpy": ([P, F, P, I], None),
    "mp_vec_aypx": ([P, F, P, I], None),
    "mp_vec_axpby": ([P, F, F, P, I], None),
    "mp_vec_axpbypcz": ([P, F, F, F, P, P, I], None),
    "mp_vec_waxpy": ([P, F, P, P, I], None),
    "mp_vec_maxpy": ([P, I, P, P, I], None),
    "mp_vec_max_pointwise_divide": ([P, P, P, I], None),
    "mp_mat_get_diagonal_markers": ([P, P, P, I], I),
    "mp_pc_jacobi_setup": ([P, I, I, I, F, P, P, P, I, P], None),
    "mp_pc_jacobi_setup_symmetric": ([P, I, P, P, P, I], None),
    "mp_pc_jacobi_apply": ([P, P, P, I], None),
    "mp_pc_sor_apply": ([P, P, P, P, P, P, P, P, P, F, F, I, I], None),
    "mp_pc_ilu_apply": ([P] * 9 + [I], None),
    "mp_pc_icc_apply": ([P] * 8 + [I], I),
    "mp_pc_ilu_numeric": ([P] * 10 + [I], I),
    "mp_pc_icc_numeric": ([P] * 12 + [I], None),
    "mp_ilu_symbolic_ilu0": ([P] * 6 + [I], I),
    "mp_ilu_symbolic": ([P] * 8 + [I, I, P, I], I),
    "mp_icc_symbolic": ([P] * 8 + [I, I, P, I, I], I),
    "mp_ilu_contiguous_lu": ([P] * 4 + [I], None),
    "mp_ordering_rcm": ([P] * 6 + [I], None),
    "mp_icc_contiguous_cholesky": ([P] * 6 + [I], None),
    "mp_ksp_solve_cg": ([I, P, P, P, P, P, P, P, P, P, P, P], None),
    "mp_ksp_solve_bcgs": ([I, P, P, P, P, P, P, P, P, P, P, P], None),
    "mp_ksp_solve_gmres": ([I] + [P] * 13, None),
    "mp_ksp_solve_fgmres": ([I] + [P] * 14, None),
}



def build() -> str:
    """Compile liboracle.so with the committed Makefile (plain gcc)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_libs = {}
_which = "parity"


def set_build(which: str) -> None:
    """Select the library every later call uses: "parity" (the default, every
    check) or "timing" (the CPU baseline's timed solves)."""
    global _which
    if which not in ("parity", "timing"):
        raise ValueError(which)
    _which = which


def lib() -> ctypes.CDLL:
    L = _libs.get(_which)
    if L is None:
        path = LIB if _which == "parity" else LIB_TIMING
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for name, (argtypes, restype) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = argtypes
            fn.restype = restype
        _libs[_which] = L
    return L


def a(arr) -> int:
    """The data address of `arr`.  The caller must keep `arr` referenced until
    the call that uses the address returns (never pass a temporary)."""
    return arr.ctypes.data


def i64(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.int64)


def f64(x) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.float64)


# ------------------------------------------------------------- PC set-up

PC_CODES = {"none": 0, "jacobi": 2, "sor": 4, "ilu": 5, "icc": 6}
SOR_FORWARD_SWEEP = 1
SOR_LOCAL_SYMMETRIC_SWEEP = 12
SOR_ZERO_INITIAL_GUESS = 16


class OraclePC:
    """The reference PC's host state (PC.py:108-148, 315-547) over the oracle."""

    def __init__(self, pc_type, irow, icol, data, *, levels=0, ordering="natural",
                 omega=1.0, fshift=0.0, symmetric=True, jacobi_type=0,
                 use_abs=False, fix_diag=True, rowl1_scale=1.0):
        self.type = pc_type
        self.irow, self.icol, self.data = i64(irow), i64(icol), f64(data)
        self.n = n = len(self.irow) - 1
        self.levels = levels
        self.ordering = ordering
        self.omega, self.fshift = float(omega), float(fshift)
        self.symmetric = symmetric
        self.keep = []
        L = lib()
        if pc_type == "jacobi":
            self.diag = np.zeros(max(n, 1))
            didx = np.zeros(max(n, 1))
            L.mp_pc_jacobi_setup(a(self.diag), jacobi_type, int(use_abs), int(fix_diag),
                                 float(rowl1_scale), a(self.irow), a(self.icol),
                                 a(self.data), n, a(didx))
            self.diagsqrt = np.zeros(max(n, 1))
            L.mp_pc_jacobi_setup_symmetric(a(self.diagsqrt), jacobi_type, a(self.irow),
                                           a(self.icol), a(self.data), n)
        elif pc_type == "sor":
            k = max(n, 1)
            self.dmark = np.zeros(k, dtype=np.int64)
            L.mp_mat_get_diagonal_markers(a(self.irow), a(self.icol), a(self.dmark), n)
            self.idiag = np.zeros(k)
            self.mdiag = np.zeros(k)
            self.sorwork = np.zeros(3 * k)
        elif pc_type in ("ilu", "icc"):
            self._build_factor()
        elif pc_type != "none":
            raise NotImplementedError(pc_type)

    def _perms(self):
        n = self.n
        if self.ordering == "rcm" and n > 0:
            perm = np.zeros(n, dtype=np.int64)
            lvl = np.zeros(n, dtype=np.int64)
            vis = np.zeros(n, dtype=np.int64)
            q = np.zeros(n, dtype=np.int64)
            lib().mp_ordering_rcm(a(perm), a(lvl), a(vis), a(q), a(self.irow), a(self.icol), n)
            r = perm
        else:
            r = np.arange(n, dtype=np.int64)
        ic = np.empty(n, dtype=np.int64)
        ic[r] = np.arange(n, dtype=np.int64)
        return r, ic

    def _build_factor(self):
        n = self.n
        L = lib()
        r, ic = self._perms()
        adiag = np.zeros(n, dtype=np.int64)
        L.mp_mat_get_diagonal_markers(a(self.irow), a(self.icol), a(adiag), n)
        scratch = np.zeros(7 * n + 8, dtype=np.int64)
        cap = max(4 * n, 4 * int(self.irow[-1]) + 4 * n, 16)
        if self.type == "ilu":
            while True:
                bi = np.zeros(n + 1, dtype=np.int64)
                bj = np.zeros(cap, dtype=np.int64)
                bjlvl = np.zeros(cap, dtype=np.int64)
                bdiag = np.zeros(n + 1, dtype=np.int64)
                if self.levels == 0 and np.array_equal(r, np.arange(n)):
                    nnz = L.mp_ilu_symbolic_ilu0(a(bi), a(bj), a(bdiag), a(adiag),
                                                 a(self.irow), a(self.icol), n)
                    contiguous = False
                else:
                    bjsrc = np.zeros(cap, dtype=np.int64)
                    nnz = L.mp_ilu_symbolic(a(bi), a(bjsrc), a(bjlvl), a(bdiag),
                                            a(self.irow), a(self.icol), a(r), a(ic),
                                            self.levels, cap, a(scratch), n)
                    contiguous = True
                if nnz >= 0:
                    if contiguous:
                        L.mp_ilu_contiguous_lu(a(bjsrc), a(bi), a(bdiag), a(bj), n)
                    break
                cap = -nnz + n
            ba = np.zeros(max(int(bdiag[0]) + 1, 1))
            rtmp = np.zeros(n)
            L.mp_pc_ilu_numeric(a(ba), a(rtmp), a(self.irow), a(self.icol), a(self.data),
                                a(bi), a(bj), a(bdiag), a(r), a(ic), n)
            self.factor = {"bi": bi, "bj": bj, "ba": ba, "bdiag": bdiag, "r": r, "c": r}
        else:
            rinv = np.empty(n, dtype=np.int64)
            rinv[r] = np.arange(n, dtype=np.int64)
            while True:
                ui = np.zeros(n + 1, dtype=np.int64)
                uj = np.zeros(cap, dtype=np.int64)
                ujlvl = np.zeros(cap, dtype=np.int64)
                udiag = np.zeros(n, dtype=np.int64)
                need = 6 * (n + 1) + 2 * cap
                if scratch.size < need:
                    scratch = np.zeros(need, dtype=np.int64)
                nnz = L.mp_icc_symbolic(a(ui), a(uj), a(ujlvl), a(udiag), a(self.irow),
                                        a(self.icol), a(r), a(rinv), self.levels, cap,
                                        a(scratch), n, int(scratch.size))
                if nnz >= 0:
                    break
                cap = -nnz
            bi = np.zeros(n + 1, dtype=np.int64)
            bdiag = np.zeros(n + 1, dtype=np.int64)
            bj = np.zeros(max(cap, int(ui[-1]) + 1), dtype=np.int64)
            bdiag[:n] = udiag[:n]
            L.mp_icc_contiguous_cholesky(a(uj), a(ui), a(bdiag), a(bi), a(bdiag), a(bj), n)
            ua = np.zeros(max(int(ui[-1]), 1))
            rtmp = np.zeros(n)
            il = np.zeros(n, dtype=np.int64)
            c2r = np.zeros(n, dtype=np.int64)
            L.mp_pc_icc_numeric(a(ua), a(rtmp), a(il), a(c2r), a(self.irow), a(self.icol),
                                a(self.data), a(bi), a(bj), a(bdiag), a(r), a(rinv), n)
            self.factor = {"bi": bi, "bj": bj, "ba": ua, "bdiag": bdiag, "r": r}

    def sor_flag(self):
        return ((SOR_LOCAL_SYMMETRIC_SWEEP if self.symmetric else SOR_FORWARD_SWEEP)
                | SOR_ZERO_INITIAL_GUESS)

    def pci(self):
        pci = np.zeros(12, dtype=np.int64)
        pci[0] = PC_CODES[self.type]
        if self.type == "jacobi":
            pci[1] = a(self.diag)
            pci[2] = a(self.diagsqrt)
        elif self.type == "sor":
            pci[1], pci[2], pci[3] = a(self.irow), a(self.icol), a(self.data)
            pci[4], pci[5], pci[6] = a(self.dmark), a(self.idiag), a(self.mdiag)
            pci[7] = a(self.sorwork)
            pci[10] = self.sor_flag()
        elif self.type in ("ilu", "icc"):
            f = self.factor
            pci[1], pci[2], pci[3], pci[4], pci[5] = (a(f["bi"]), a(f["bj"]), a(f["ba"]),
                                                      a(f["bdiag"]), a(f["r"]))
            if self.type == "ilu":
                pci[6] = a(f["c"])
        return pci

    def apply(self, x):
        """PC.apply (PC.py:590-633) on a host array."""
        n = self.n
        x = f64(x)
        y = np.zeros(n)
        L = lib()
        if self.type == "none":
            y[:] = x
        elif self.type == "jacobi":
            L.mp_pc_jacobi_apply(a(y), a(x), a(self.diag), n)
        elif self.type == "sor":
            L.mp_pc_sor_apply(a(x), a(y), a(self.irow), a(self.icol), a(self.data),
                              a(self.dmark), a(self.idiag), a(self.mdiag), a(self.sorwork),
                              self.omega, self.fshift, self.sor_flag(), n)
        elif self.type == "ilu":
            f = self.factor
            tmp = np.zeros(n)
            L.mp_pc_ilu_apply(a(x), a(y), a(tmp), a(f["bi"]), a(f["bj"]), a(f["ba"]),
                              a(f["bdiag"]), a(f["r"]), a(f["c"]), n)
        else:
            f = self.factor
            scratch = np.zeros(n)
            L.mp_pc_icc_apply(a(x), a(y), a(f["bi"]), a(f["bj"]), a(f["ba"]), a(f["bdiag"]),
                              a(f["r"]), a(scratch), n)
        return y


# ------------------------------------------------------------- KSP solve

NORM_NONE, NORM_PRECONDITIONED, NORM_UNPRECONDITIONED, NORM_NATURAL = 1, 2, 3, 4


def solve(ksp_type, irow, icol, data, b, *, pc_type="none", x0=None, rtol=1e-5,
          atol=1e-50, divtol=1e4, max_it=None, restart=30, normtype=0, pc_side=0,
          min_it=0, chknorm=-1, haptol=1e-30, breakdowntol=0.1, orthog=0, cgstype=0,
          pc=None, **pc_opts):
    """KSP.solve (KSP.py:367-449) through the oracle; returns a dict with
    x, its, reason, rnorm and the residual history up to its."""
    irow, icol, data = i64(irow), i64(icol), f64(data)
    n = len(irow) - 1
    b = f64(b).copy()
    if pc is None:
        pc = OraclePC(pc_type, irow, icol, data, **pc_opts)
    convmaxits = 0
    if max_it is None:
        max_it = 1000
    else:
        convmaxits = 1
    guess_zero = 1 if x0 is None else 0
    x = np.zeros(n) if x0 is None else f64(x0).copy()
    if normtype == 0:
        normtype = NORM_PRECONDITIONED
    cfg = np.zeros(16 + max_it + 2)
    cfg[0], cfg[1], cfg[2], cfg[3], cfg[4] = rtol, atol, divtol, haptol, breakdowntol
    cfgi = np.zeros(16, dtype=np.int64)
    cfgi[:10] = [normtype, pc_side, guess_zero, min_it, chknorm, convmaxits, max_it,
                 restart, orthog, cgstype]
    # KSP.py:496-507 _rhs_norm for a nonzero guess
    rhs = 0.0
    if not guess_zero and normtype != NORM_NONE:
        if normtype == NORM_UNPRECONDITIONED or pc_side == 1:
            rhs = float(np.linalg.norm(b))
        else:
            z = pc.apply(b)
            if normtype == NORM_PRECONDITIONED:
                rhs = float(np.linalg.norm(z))
            else:
                rhs = math.sqrt(abs(float(z @ b)))
    cfg[12] = rhs
    cfg[14] = 0.0
    cfgi[12] = 0 if guess_zero else 1
    pci = pc.pci()
    pcf = np.array([pc.omega, pc.fshift])
    pstmp = np.zeros(max(n, 1))
    L = lib()
    if ksp_type in ("gmres", "fgmres"):
        mk = restart
        hs = np.zeros((mk + 2) * (mk + 1) + (mk + 1) ** 2 + 2 * (mk + 1) + 2 * (mk + 2))
        work = np.zeros(2 * n)
        vv = np.zeros((mk + 1) * n)
        if ksp_type == "gmres":
            L.mp_ksp_solve_gmres(n, a(irow), a(icol), a(data), a(pci), a(pcf), a(pstmp),
                                 a(work), a(vv), a(hs), a(cfg), a(cfgi), a(b), a(x))
        else:
            prevec = np.zeros((mk + 2) * n)
            L.mp_ksp_solve_fgmres(n, a(irow), a(icol), a(data), a(pci), a(pcf), a(pstmp),
                                  a(work), a(vv), a(prevec), a(hs), a(cfg), a(cfgi), a(b),
                                  a(x))
    elif ksp_type in ("cg", "bcgs"):
        work = np.zeros(7 * n)
        fn = L.mp_ksp_solve_cg if ksp_type == "cg" else L.mp_ksp_solve_bcgs
        fn(n, a(irow), a(icol), a(data), a(pci), a(pcf), a(pstmp), a(work), a(cfg), a(cfgi),
           a(b), a(x))
    else:
        raise NotImplementedError(ksp_type)
    its = int(cfgi[10])
    return {"x": x, "its": its, "reason": int(cfgi[11]), "rnorm": float(cfg[7]),
            "history": cfg[9:9 + its + 1].copy()}
