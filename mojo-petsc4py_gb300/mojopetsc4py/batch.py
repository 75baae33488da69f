"""Batched CG: hundreds of independent SPD systems with several right-hand
sides each, solved together on the GPU (include/gpetsc.h, gp_batch_*).

    solver = BatchedCG([(indptr, indices, data), ...], nrhs=16)
    X, info = solver.solve(B, pc="jacobi", precision="fp64", rtol=1e-8)

`B` stacks the systems' right-hand sides row-wise: an (sum n_s, nrhs) FP64
array, either on the host (anything numpy reads) or on the device (anything
with __cuda_array_interface__: a CUDA torch tensor, a CuPy array, the
library's own DeviceArray).  `X` has the same shape: a numpy array for a host
`B`, a tensor of the same kind for a torch `B`, else a DeviceArray.  Each (system, column) pair follows the CG recurrence of
KSPSolve_CG (src/ksp.mojo:271-389) with its own stopping test.
precision="fp32" solves each pair with an FP32 inner CG inside FP64
iterative refinement until the true FP64 residual meets rtol.

`shard_systems` splits a batch across ranks (one GPU each) by a greedy
balance of nnz * nrhs; the systems are independent, so a sharded run needs
no collective beyond gathering the results.
"""
from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import _device as dev
from ._lib import check, lib

_PC = {"none": 0, "jacobi": 2, "icc": 6}
_PREC = {"fp64": 0, "fp32": 1}


class BatchOptions(ctypes.Structure):
    _fields_ = [("pc_type", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("max_it", ctypes.c_int32), ("max_outer", ctypes.c_int32),
                ("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("divtol", ctypes.c_double), ("inner_rtol", ctypes.c_double)]


def stack_systems(systems):
    """Concatenate (indptr, indices, data) triples into one block-diagonal CSR.
    Returns (sys_rows, indptr, indices, data) as int64/float64 arrays."""
    sizes = [len(ip) - 1 for ip, _, _ in systems]
    sys_rows = np.zeros(len(systems) + 1, dtype=np.int64)
    sys_rows[1:] = np.cumsum(sizes)
    nnz = [int(ip[-1]) for ip, _, _ in systems]
    offs = np.concatenate([[0], np.cumsum(nnz)]).astype(np.int64)
    indptr = np.zeros(int(sys_rows[-1]) + 1, dtype=np.int64)
    indices = np.empty(int(offs[-1]), dtype=np.int64)
    data = np.empty(int(offs[-1]), dtype=np.float64)
    for s, (ip, ix, v) in enumerate(systems):
        r0, r1 = int(sys_rows[s]), int(sys_rows[s + 1])
        indptr[r0 + 1:r1 + 1] = np.asarray(ip[1:], dtype=np.int64) + offs[s]
        indices[offs[s]:offs[s + 1]] = np.asarray(ix, dtype=np.int64) + r0
        data[offs[s]:offs[s + 1]] = v
    return sys_rows, indptr, indices, data


def shard_systems(costs, world: int):
    """Greedy longest-processing-time split of systems (cost = nnz * nrhs)
    over `world` ranks: returns one sorted list of system indices per rank."""
    order = sorted(range(len(costs)), key=lambda s: (-costs[s], s))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for s in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(s)
        load[r] += costs[s]
    return [sorted(x) for x in out]


class BatchedCG:
    def __init__(self, systems, nrhs: int = 16, autotune: bool = True):
        if nrhs not in (1, 2, 4, 8, 16):
            raise ValueError("nrhs must be 1, 2, 4, 8 or 16")
        dev.require_device()
        self.nrhs = nrhs
        self.sys_rows, indptr, indices, data = stack_systems(systems)
        self.nsys = len(systems)
        self.n = int(self.sys_rows[-1])
        h = ctypes.c_void_p()
        check(lib().gp_batch_create(ctypes.byref(h), self.nsys, self.sys_rows.ctypes.data,
                                    indptr.ctypes.data, indices.ctypes.data,
                                    data.ctypes.data if len(data) else None, nrhs,
                                    dev.stream_ptr()))
        self._h = h.value
        if autotune:
            check(lib().gp_batch_autotune(self._h, dev.stream_ptr()))

    def __del__(self):
        try:
            lib().gp_batch_destroy(self._h)
        except Exception:
            pass

    def _tuning(self, precision: int):
        bl, vr, tr = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        us = ctypes.c_double()
        check(lib().gp_batch_tuning(self._h, precision, ctypes.byref(bl), ctypes.byref(vr),
                                    ctypes.byref(tr), ctypes.byref(us)))
        return {"block": bl.value, "columns_per_thread": vr.value, "tile_rows": tr.value,
                "spmm_us": us.value}

    @property
    def tuning(self):
        """The autotuner's choice for the FP64 sparse pass."""
        return self._tuning(0)

    @property
    def tuning32(self):
        """The autotuner's choice for the FP32 sparse pass."""
        return self._tuning(1)

    def solve(self, B, pc: str = "jacobi", precision: str = "fp64", rtol: float = 1e-8,
              atol: float = 1e-50, divtol: float = 1e4, max_it: int = 10000,
              max_outer: int = 20, inner_rtol: float = 1e-4, out=None):
        if pc not in _PC or precision not in _PREC:
            raise NotImplementedError(f"batched CG supports pc {sorted(_PC)} and precision "
                                      f"{sorted(_PREC)}")
        shape = (self.n, self.nrhs)
        bad = ValueError(f"B must be float64 of shape ({self.n}, {self.nrhs})")
        view = dev.device_view(B)
        host = view is None
        if host:
            Bh = np.ascontiguousarray(B, dtype=np.float64)
            if Bh.shape != shape:
                raise bad
            Bd = dev.from_host(Bh)
            bp = Bd.ptr
        else:
            bp, bshape, bdtype = view
            if bshape != shape or bdtype != np.float64:
                raise bad
        if out is not None:
            X = out
            oview = dev.device_view(out)
            if oview is None or oview[1] != shape or oview[2] != np.float64:
                raise ValueError("out must be a float64 device array of B's shape")
            xp = oview[0]
        else:
            X = dev.DeviceArray(shape)
            xp = X.ptr
            if not host and type(B).__module__.split(".")[0] == "torch":
                X = sys.modules["torch"].as_tensor(X, device=B.device)
        o = BatchOptions()
        lib().gp_batch_options_default(ctypes.byref(o))
        o.pc_type, o.precision = _PC[pc], _PREC[precision]
        o.max_it, o.max_outer = int(max_it), int(max_outer)
        o.rtol, o.atol, o.divtol, o.inner_rtol = rtol, atol, divtol, inner_rtol
        npairs = self.nsys * self.nrhs
        its = np.zeros(npairs, dtype=np.int64)
        reason = np.zeros(npairs, dtype=np.int32)
        relres = np.zeros(npairs, dtype=np.float64)
        passes = ctypes.c_int32()
        check(lib().gp_batch_solve_cg(self._h, ctypes.byref(o), bp, xp,
                                      its.ctypes.data, reason.ctypes.data, relres.ctypes.data,
                                      ctypes.byref(passes), dev.stream_ptr()))
        pshape = (self.nsys, self.nrhs)
        info = {"its": its.reshape(pshape), "reason": reason.reshape(pshape),
                "relres": relres.reshape(pshape), "passes": passes.value}
        if host and out is None:
            return X.to_host(), info
        return X, info


def assemble_shards(shards, parts, sizes, nrhs: int):
    """Reassemble the ranks' results of a sharded batch in system order.

    shards  one list of system indices per rank (ascending, as shard_systems
            returns them)
    parts   one dict per rank: "X" -- its systems' solutions stacked row-wise,
            shape (sum of their sizes, nrhs); "its", "reason", "relres" --
            shape (len(shard), nrhs)
    sizes   rows of every system of the whole batch
    Returns (X of shape (sum sizes, nrhs), info with its / reason / relres of
    shape (nsys, nrhs)).  Raises ValueError unless every system appears in
    exactly one shard with a part of matching shape."""
    nsys = len(sizes)
    offs = np.zeros(nsys + 1, dtype=np.int64)
    offs[1:] = np.cumsum(sizes)
    if len(shards) != len(parts):
        raise ValueError("one part per shard expected")
    seen = np.zeros(nsys, dtype=np.int64)
    X = np.empty((int(offs[-1]), nrhs), dtype=np.float64)
    its = np.zeros((nsys, nrhs), dtype=np.int64)
    reason = np.zeros((nsys, nrhs), dtype=np.int32)
    relres = np.zeros((nsys, nrhs), dtype=np.float64)
    for shard, part in zip(shards, parts):
        rows = int(sum(sizes[s] for s in shard))
        if np.shape(part["X"]) != (rows, nrhs) or np.shape(part["its"]) != (len(shard), nrhs):
            raise ValueError("part shape does not match its shard")
        r = 0
        for k, s in enumerate(shard):
            m = int(sizes[s])
            X[offs[s]:offs[s] + m] = part["X"][r:r + m]
            its[s], reason[s], relres[s] = part["its"][k], part["reason"][k], part["relres"][k]
            seen[s] += 1
            r += m
    if not np.all(seen == 1):
        raise ValueError("every system must belong to exactly one shard")
    return X, {"its": its, "reason": reason, "relres": relres}


def sharded_solve(systems, B, rank: int, world: int, gather, nrhs: int = 16,
                  autotune: bool = True, **solve_kw):
    """Solve this rank's shard of a batch and gather the results on rank 0.

    Every rank passes the whole batch (`systems`, and `B` as an
    (sum n_s, nrhs) host array); shard_systems decides the split the same
    way on every rank, so no message is needed before the solve.  `gather`
    is a host-side collective: gather(obj) returns the list of all ranks'
    objects on rank 0 and None elsewhere (a gloo gather_object, or
    `lambda o: [o]` for one rank).  Returns (solver, X, info) on rank 0 --
    X and info for the whole batch in system order -- and (solver, None,
    None) elsewhere; the solver is this rank's, for timing repeat solves."""
    sizes = [len(ip) - 1 for ip, _, _ in systems]
    costs = [int(ip[-1]) * nrhs for ip, _, _ in systems]
    shards = shard_systems(costs, world)
    mine = shards[rank]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    if mine:
        solver = BatchedCG([systems[s] for s in mine], nrhs=nrhs, autotune=autotune)
        Bm = np.concatenate([B[offs[s]:offs[s + 1]] for s in mine])
        Xm, info = solver.solve(Bm, **solve_kw)
    else:  # more ranks than systems
        solver, Xm = None, np.zeros((0, nrhs))
        info = {"its": np.zeros((0, nrhs), dtype=np.int64),
                "reason": np.zeros((0, nrhs), dtype=np.int32),
                "relres": np.zeros((0, nrhs))}
    parts = gather({"X": Xm, "its": info["its"], "reason": info["reason"],
                    "relres": info["relres"]})
    if parts is None:
        return solver, None, None
    X, full = assemble_shards(shards, parts, sizes, nrhs)
    return solver, X, full
