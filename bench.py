"""Benchmark: solve time to rtol 1e-10 on the 3-D 7-point Poisson operator,
128^3 (n = 2,097,152, nnz = 14,581,760), through the PETSc-compatible API on
one GB300.

One step = one KSP.solve of that system with CG + Jacobi (b uniform[-1, 1],
seed 5, x0 = 0, rtol 1e-10, atol 1e-50, max_it 10000).  The matrix (217 MB)
is larger than the 129 MB L2, so consecutive solves stream it from HBM.

  value   device-resident solve time (b, x and the operator already in HBM)
  e2e     the same solve through the public API with host arrays: the step
          uploads b from host memory, solves, and reads x back
  roofline  the SpMV kernel, timed with CUDA events over 20 back-to-back
          launches after a 512 MB read (the matrix, 188 MB with its 16-bit
          column offsets, is larger than L2, so every launch streams it from
          HBM), algorithmic bytes (8 + c) nnz + 4 (n+1) + 16 n per launch, c
          the column bytes the kernel reads (2 or 4)
  cpu_baseline  the CPU oracle (a single-threaded restatement of the
          reference's algorithm) on the same system: one whole solve, timed

`--impl reference` times the reference's CPU path (the oracle restatement;
the Mojo reference cannot be built here) on the same workload and prints the
same JSON line with "impl": "reference": every step is one whole solve.

Multi-GPU (`--gpus N`; started under torchrun, or relaunched under it when
WORLD_SIZE is unset): every rank solves its own replica of the plain system
(the path is sequential; there is no data-path collective), with a barrier
and the max over ranks around the timed region; the batched form splits its
systems over the ranks and gathers only the results.
"""

from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "mojo-petsc4py_gb300"))

K3 = 128
RTOL = 1e-10
MAX_IT = 10000
METRIC = "solve ms to rtol 1e-10 (3-D 7-pt Poisson 128^3, CG+Jacobi, FP64)"


# the plain methods of the 128^3 configuration: (ksp type, pc type, pc options)
METHODS = {"cg+jacobi": ("cg", "jacobi", {}), "cg+icc(0)": ("cg", "icc", {}),
           "gmres(30)+ilu(0)": ("gmres", "ilu", {}), "bcgs+sor(1.2)": ("bcgs", "sor", {"omega": 1.2})}


def config(world):
    """The workload, identical in both arms' JSON lines."""
    return {"workload": "poisson3d-7pt-128^3 cg+jacobi rtol 1e-10", "n": K3 ** 3,
            "nnz": 7 * K3 ** 3 - 6 * K3 ** 2, "method": "cg+jacobi", "rtol": RTOL,
            "atol": 1e-50, "max_it": MAX_IT, "rhs": "uniform[-1, 1], numpy default_rng(5)",
            "x0": "zero", "l2": "inputs larger than L2 (matrix 217 MB)",
            "parallelism": f"replicas x{world}"}


def cpu_info():
    """Host CPU model and logical core count."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        import platform

        model = platform.processor() or platform.machine()
    return {"cpu_model": model, "os_cpu_count": os.cpu_count()}


def problem():
    from mojopetsc4py import gallery

    ip, ix, v = gallery.laplacian_3d(K3)
    n = len(ip) - 1
    b = np.random.default_rng(5).uniform(-1.0, 1.0, n)
    return ip, ix, v, b


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(name):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    """(world, rank, local rank, process group or None) from the torchrun
    environment.  NCCL carries the default group on GPUs; a gloo group
    carries host objects (the batched form's results)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            tdist.init_process_group("gloo")
        pg = tdist
    return world, rank, local, pg


_GLOO = None


def host_group(pg):
    """A gloo group over all ranks for host-side objects."""
    global _GLOO
    if pg is None:
        return None
    if _GLOO is None:
        _GLOO = pg.new_group(backend="gloo") if pg.get_backend() != "gloo" else pg.group.WORLD
    return _GLOO


def barrier(pg):
    if pg is not None:
        pg.barrier(group=host_group(pg))


def max_over_ranks(pg, value):
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX, group=host_group(pg))
    return float(t.item())


def gather_to_root(pg, obj):
    """List of every rank's `obj` on rank 0 (None elsewhere); [obj] alone."""
    if pg is None:
        return [obj]
    out = [None] * pg.get_world_size() if pg.get_rank() == 0 else None
    pg.gather_object(obj, out, dst=0, group=host_group(pg))
    return out


# ------------------------------------------------------------------ CPU leg
# the oracle's timing build (FMA contraction, -O3; -march=native is not used
# because the host code must build the same on x86_64 and aarch64)
ORACLE_TIMING_BUILD = "gcc -O3 -ffp-contract=fast -fno-fast-math, 1 thread"


def oracle_cg_jacobi(ip, ix, v, b, max_it=MAX_IT, build="timing"):
    """One timed CG + Jacobi solve of the oracle: (seconds, result).  The
    Jacobi set-up is outside the timing, as the reference's bench.py keeps
    set-up out of its solve timings.  `build` "timing" (the CPU baseline) or
    "parity" (the checker, whose iterate the GPU results are compared with)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.set_build(build)
    try:
        O.lib()
        ip, ix, v, b = O.i64(ip), O.i64(ix), O.f64(v), O.f64(b)
        pc = O.OraclePC("jacobi", ip, ix, v)
        t0 = time.perf_counter()
        r = O.solve("cg", ip, ix, v, b, pc=pc, rtol=RTOL, atol=1e-50, divtol=1e30,
                    max_it=max_it)
        return time.perf_counter() - t0, r
    finally:
        O.set_build("parity")


def run_reference(args, world, rank, pg):
    """The reference's CPU path (the oracle restatement, single-threaded as
    the reference library is): every timed step is one whole CG + Jacobi
    solve of the benchmark system; each warm-up step a 40-iteration solve,
    which pages in the matrix and vectors."""
    if rank != 0:
        return
    ip, ix, v, b = problem()
    for _ in range(args.warmup):
        oracle_cg_jacobi(ip, ix, v, b, max_it=40)
    per, its, reason = [], None, None
    for _ in range(args.steps):
        dt, r = oracle_cg_jacobi(ip, ix, v, b)
        per.append(dt * 1e3)
        its, reason = r["its"], r["reason"]
    ms = float(np.mean(per))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(world),
        "result": {"iterations": its, "reason": reason,
                   "median_ms": round(float(np.median(per)), 3),
                   "best_of_3_ms": round(float(min(per[:3])), 3)},
        "cpu_baseline": {"value": round(ms, 3), "unit": "ms", "cores": 1, "kind": "port",
                         "sample": f"whole {its}-iteration CG+Jacobi solves, mean of "
                                   f"{args.steps} (warm-up: {args.warmup} solves of 40 "
                                   "iterations)", "build": ORACLE_TIMING_BUILD,
                         **cpu_info()},
        "e2e": {"value": round(ms, 3), "unit": "ms", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
def build_solver(PETSc, A, ksp_type, pc_type, **opts):
    pc = PETSc.PC().create()
    pc.setType(pc_type)
    if pc_type == "sor":
        pc.setSOROmega(opts.get("omega", 1.0))
    pc.setOperators(A)
    ksp = PETSc.KSP().create()
    ksp.setPC(pc)
    ksp.setType(ksp_type)
    ksp.setOperators(A)
    ksp.setTolerances(rtol=RTOL, atol=1e-50, divtol=1e30, max_it=MAX_IT)
    if ksp_type in ("gmres", "fgmres"):
        ksp.setGMRESRestart(30)
    return ksp


def time_solves(torch, ksp, bv, xv, steps, per_solve=None):
    """Mean ms per solve over `steps` back-to-back solves (one event pair
    around all of them); with a list in `per_solve`, each solve's own ms
    (an event between consecutive solves) is appended to it."""
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    torch.cuda.synchronize()
    evs[0].record()
    for k in range(steps):
        ksp.solve(bv, xv)
        evs[k + 1].record()
    torch.cuda.synchronize()
    if per_solve is not None:
        per_solve.extend(a.elapsed_time(b) for a, b in zip(evs[:-1], evs[1:]))
    return evs[0].elapsed_time(evs[-1]) / steps


def spmv_roofline(torch, PETSc, A, n, nnz, launches=20):
    import ctypes

    from mojopetsc4py import _device as dev
    from mojopetsc4py._lib import check, lib

    x = PETSc.Vec().createWithArray(np.random.default_rng(3).normal(size=n))
    y = PETSc.Vec().createSeq(n)
    h = A._device()
    # flush by reading 512 MB, so L2 holds clean lines of another buffer and the
    # kernel pays no write-back of a flush
    flush = torch.ones(int(512 * 2**20 // 8), dtype=torch.float64, device="cuda")
    xp, yp = x._dptr(), y._optr()
    st = dev.stream_ptr()
    for _ in range(3):
        check(lib().gp_mat_mult(h, xp, yp, st))
    # `launches` back-to-back launches between two events: the matrix (217 MB)
    # is larger than the 129 MB L2, so every launch streams it from HBM, and
    # no host gap can fall inside the timed region
    flush.sum()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(launches):
        check(lib().gp_mat_mult(h, xp, yp, st))
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / launches
    ib = spmv_index_bytes(h)
    algo = (8 + ib) * nnz + 4 * (n + 1) + 8 * n + 8 * n
    return algo, t, ib


def spmv_index_bytes(h):
    """Column bytes the SpMV reads per entry: 2 (row-relative 16-bit offsets)
    or 4 (32-bit indices)."""
    import ctypes

    from mojopetsc4py._lib import check, lib

    b = ctypes.c_int32()
    check(lib().gp_mat_spmv_index_bytes(h, ctypes.byref(b)))
    return b.value


def run_spmv_only(args):
    """SpMV launches alone on the 7-point matrix of a k^3 grid (k =
    --spmv-grid, the benchmark's 128 by default; the profiling target), or
    with --spmv-hubs on the skewed-row operator of the bandwidth form (a path
    graph of 2^20 rows with 8 hub rows of ~100k entries: the row-stream
    SpMV and, in the FMA arithmetic, the hubs summed by segments)."""
    import torch

    from mojopetsc4py import PETSc

    from mojopetsc4py import gallery

    if args.spmv_hubs:
        ip, ix, v = gallery.hub_laplacian(1 << 20, 8, 100_000)
    else:
        ip, ix, v = gallery.laplacian_3d(args.spmv_grid)
    n, nnz = len(ip) - 1, int(ip[-1])
    A = PETSc.Mat().createSeqAIJ((n, n), nnz=None if args.spmv_hubs else 7)
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    algo, t, _ = spmv_roofline(torch, PETSc, A, n, nnz, launches=args.steps)
    print(json.dumps({"kernel": "k_spmv", "matrix": "hubs_2^20" if args.spmv_hubs else
                      f"poisson3d_{args.spmv_grid}^3", "n": n, "nnz": nnz,
                      "algorithmic_bytes": algo, "launch_us": t * 1e6,
                      "achieved_gbs": algo / t / 1e9}), flush=True)


def run_ours(args, world, rank, local, pg):
    import torch

    torch.cuda.set_device(local)
    from mojopetsc4py import PETSc

    ip, ix, v, b = problem()
    n, nnz = len(b), int(ip[-1])
    A = PETSc.Mat().createSeqAIJ((n, n), nnz=7)
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    kt0, pt0, po0 = METHODS[args.method]
    ksp = build_solver(PETSc, A, kt0, pt0, **po0)
    bv = PETSc.Vec().createWithArray(b)
    xv = PETSc.Vec().createSeq(n)
    for _ in range(max(args.warmup, 3)):
        ksp.solve(bv, xv)
    its, reason = ksp.getIterationNumber(), ksp.getConvergedReason()
    trips, top, body = ksp.getLaunchStats()

    # ---- timed region: device-resident solves
    barrier(pg)
    torch.cuda.synchronize()
    per_solve = []
    with Clocks(local) as clk:
        ms = time_solves(torch, ksp, bv, xv, args.steps, per_solve)
    barrier(pg)
    ms = max_over_ranks(pg, ms)
    clocks = clk.summary()

    # ---- end to end through the public API with host arrays
    xh = xv.getArray().copy()
    barrier(pg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bv.setArray(b)
        ksp.solve(bv, xv)
        xh = xv.getArray()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
    e2e_ms = max_over_ranks(pg, e2e_ms)
    resid = float(np.linalg.norm(b - _csr_matvec(ip, ix, v, xh)) / np.linalg.norm(b))

    # ---- SpMV roofline (kernel alone, L2 flushed before each launch)
    algo, t_spmv, spmv_ib = spmv_roofline(torch, PETSc, A, n, nnz)
    peak, peak_kind = peaks()
    achieved = algo / t_spmv / 1e9
    traffic = profiled_traffic("spmv_fp64_poisson3d_128.md")

    # ---- the other plain methods of this configuration (fewer repetitions)
    methods = {"cg+jacobi": {"ms": round(ms, 3), "its": its, "reason": reason,
                             "median_ms": round(float(np.median(per_solve)), 3),
                             "best_of_3_ms": round(float(min(per_solve[:3])), 3)}}
    if not args.quick:
        for name, kt, pt, extra in (("cg+icc(0)", "cg", "icc", {}),
                                    ("gmres(30)+ilu(0)", "gmres", "ilu", {}),
                                    ("bcgs+sor(1.2)", "bcgs", "sor", {"omega": 1.2})):
            k2 = build_solver(PETSc, A, kt, pt, **extra)
            x2 = PETSc.Vec().createSeq(n)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            k2.setUp()
            torch.cuda.synchronize()
            setup_ms = (time.perf_counter() - t0) * 1e3
            k2.solve(bv, x2)
            m2 = time_solves(torch, k2, bv, x2, 2)
            methods[name] = {"ms": round(m2, 3), "its": k2.getIterationNumber(),
                             "reason": k2.getConvergedReason(),
                             "pc_setup_ms": round(setup_ms, 2)}
        # the headline solve in the two other arithmetics: exact (rounded
        # products and sums, parallel tree reductions) and ordered (the
        # reference's blocked reduction order: a checking form whose iterate
        # is compared with the oracle's bit for bit below)
        from mojopetsc4py import _lib as gplib

        other = {}
        for mode, reps in (("exact", 3), ("ordered", 1)):
            gplib.set_arithmetic(mode)
            try:
                k3 = build_solver(PETSc, A, "cg", "jacobi")
                x3 = PETSc.Vec().createSeq(n)
                k3.solve(bv, x3)  # capture
                m3 = time_solves(torch, k3, bv, x3, reps)
                other[mode] = {"ms": round(m3, 3), "its": k3.getIterationNumber(),
                               "reason": k3.getConvergedReason(),
                               "x": x3.getArray().copy()}
            finally:
                gplib.set_arithmetic("fma")
        methods["cg+jacobi"]["other_arithmetics"] = other

    # ---- the three further forms on their own workloads (N = 1)
    forms = None
    if rank == 0 and world == 1 and not args.quick and not args.no_forms:
        forms = {}
        for name, fn in (("mixed", form_mixed), ("batched", form_batched),
                         ("adjoint", form_adjoint), ("bandwidth", form_bandwidth)):
            try:
                forms[name] = fn(torch, PETSc)
            except Exception as e:  # reported, never hidden
                forms[name] = {"error": f"{type(e).__name__}: {e}"}

    # ---- the batched form split over the ranks (N > 1; every rank takes part)
    if world > 1 and not args.quick and not args.no_forms:
        try:
            sharded = form_batched_sharded(torch, rank, world, pg)
        except Exception as e:  # reported, never hidden
            sharded = {"error": f"{type(e).__name__}: {e}"}
        forms = {"batched_sharded": sharded}

    # ---- CPU baseline (rank 0 at N = 1 only): one whole solve of the oracle
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dt, rt = oracle_cg_jacobi(ip, ix, v, b)
        cpu = {"value": round(dt * 1e3, 3), "unit": "ms", "cores": 1, "kind": "port",
               "sample": f"one whole {rt['its']}-iteration CG+Jacobi solve of the same system "
                         "on this host", "build": ORACLE_TIMING_BUILD, **cpu_info()}
        # parity of the timed solves against the oracle's parity build, same
        # inputs (untimed)
        _, rc = oracle_cg_jacobi(ip, ix, v, b, build="parity")
        rx = np.asarray(rc["x"])
        methods["cg+jacobi"]["vs_oracle"] = {
            "oracle_its": int(rc["its"]), "oracle_reason": int(rc["reason"]),
            "fma_rel_diff": float(np.linalg.norm(xh - rx) / np.linalg.norm(rx))}
        for mode, r in methods["cg+jacobi"].get("other_arithmetics", {}).items():
            r["rel_diff_vs_oracle"] = float(np.linalg.norm(r["x"] - rx) / np.linalg.norm(rx))
            r["bit_identical_to_oracle"] = bool(np.array_equal(r["x"], rx))
    for r in methods["cg+jacobi"].get("other_arithmetics", {}).values():
        r.pop("x", None)

    if rank != 0:
        return
    if args.method != "cg+jacobi":
        print(json.dumps({"method": args.method, "ms": round(ms, 3), "its": its,
                          "reason": reason, "note": "profiling run, not the benchmark"}),
              flush=True)
        return
    # whole-job figure: every rank solves one replica per step, so the job
    # completes `world` solves in the max-over-ranks step time
    line = {
        "metric": METRIC, "value": round(ms / world, 3), "unit": "ms", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 3),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": config(world),
        "result": {"iterations": its, "reason": reason, "true_rel_residual": resid,
                   "arithmetic": "fma"},
        "e2e": {"value": round(e2e_ms / world, 3), "unit": "ms", "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n + 1024},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic,
                     "kernel": "k_spmv (CSR fp64, int32 row pointers, "
                               + ("16-bit row-relative column offsets)" if spmv_ib == 2
                                  else "int32 columns)"),
                     "algorithmic_bytes": algo, "launch_us": round(t_spmv * 1e6, 2),
                     "peak_kind": f"{peak_kind} hbm_gbs"},
        "cpu_baseline": cpu,
        # counted from the captured graph; None when the loop is host-driven
        # (GPETSC_KSP_GRAPH=0, profiling runs)
        "gpu_launches": int(args.steps * (top + trips * body)) if top >= 0 else None,
        "clocks": clocks,
        "methods": methods,
        "forms": forms,
    }
    print(json.dumps(line), flush=True)


def _sync_ms(torch, fn, reps):
    """Mean wall ms of fn() over reps calls, device synchronised around each."""
    out = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        out.append((time.perf_counter() - t0) * 1e3)
    return float(np.mean(out))


BATCH_SYSTEMS = 512


def form_batched(torch, PETSc, plain_columns=1):
    """Batched CG on 512 RGG Laplacians x 16 right-hand sides (rtol 1e-8):
    Jacobi in the FP64 and FP32-inner-refined forms and IC(0) in FP64, one
    captured solve each, against the plain single-system FP64 path (one KSP
    CG + Jacobi solve per pair) measured on every system for the first
    `plain_columns` columns."""
    from mojopetsc4py import gallery
    from mojopetsc4py.batch import BatchedCG

    t0 = time.perf_counter()
    systems = gallery.rgg_batch(BATCH_SYSTEMS, seed=11)
    gen_s = time.perf_counter() - t0
    sizes = np.array([len(ip) - 1 for ip, _, _ in systems])
    n = int(sizes.sum())
    nnz = int(sum(int(ip[-1]) for ip, _, _ in systems))
    B = torch.randn(n, 16, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(12))
    t0 = time.perf_counter()
    solver = BatchedCG(systems, nrhs=16, autotune=True)
    setup_s = time.perf_counter() - t0
    out = {"config": f"{BATCH_SYSTEMS} RGG Laplacians (n log-uniform in [1024, 65536], mean "
                     "degree 8, weights U[0.5, 2], shift 1e-2) x 16 RHS N(0,1), CG, rtol 1e-8",
           "systems": BATCH_SYSTEMS, "rhs": 16, "rows": n, "nnz": nnz, "tuning": solver.tuning,
           "tuning_fp32": solver.tuning32, "generate_s": round(gen_s, 1),
           "setup_s": round(setup_s, 1)}
    X = torch.empty_like(B)
    # fp64 at rtol 1e-8 stops on the preconditioned norm (its true residual is
    # larger); fp64 at 1e-10 reaches the true 1e-8 the refined fp32 form meets
    for key, pc, prec, rt in (("fp64", "jacobi", "fp64", 1e-8),
                              ("fp64_rtol_1e-10", "jacobi", "fp64", 1e-10),
                              ("fp32_inner_fp64_refined", "jacobi", "fp32", 1e-8),
                              ("fp64_icc0", "icc", "fp64", 1e-8)):
        t0 = time.perf_counter()
        solver.solve(B, pc=pc, precision=prec, rtol=rt, out=X)  # set-up, capture, warm
        first_s = time.perf_counter() - t0
        ms = _sync_ms(torch, lambda: solver.solve(B, pc=pc, precision=prec, rtol=rt, out=X), 2)
        _, info = solver.solve(B, pc=pc, precision=prec, rtol=rt, out=X)
        out[key] = {
            "ms": round(ms, 2), "max_its": int(info["its"].max()),
            "mean_its": round(float(info["its"].mean()), 1),
            "max_true_rel_residual": float(info["relres"].max()),
            "converged_pairs": int((info["reason"] > 0).sum()), "passes": info["passes"]}
        if pc == "icc":
            out[key]["pc_setup_and_first_solve_s"] = round(first_s, 1)
    # plain FP64 path: one KSP solve per (system, column) on every system
    Bh = B.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    total_ms, solves = 0.0, 0
    for s in range(len(systems)):
        ip, ix, v = systems[s]
        m = len(ip) - 1
        A = PETSc.Mat().createSeqAIJ((m, m))
        A.setValuesCSR(ip, ix, v)
        A.assemble()
        ksp = build_solver(PETSc, A, "cg", "jacobi")
        ksp.setTolerances(rtol=1e-8, atol=1e-50, max_it=10000)
        xv = PETSc.Vec().createSeq(m)
        bv = PETSc.Vec().createWithArray(Bh[offs[s]:offs[s] + m, 0].copy())
        ksp.solve(bv, xv)  # set-up and capture, untimed
        for c in range(plain_columns):
            bv.setArray(Bh[offs[s]:offs[s] + m, c].copy())
            total_ms += _sync_ms(torch, lambda: ksp.solve(bv, xv), 1)
            solves += 1
    all_ms = total_ms * (16 / plain_columns)
    out["plain_fp64_single_system"] = {
        "measured_solves": solves, "measured_ms": round(total_ms, 1),
        "ms_all_pairs": round(all_ms, 1),
        "how": f"KSP cg+jacobi, one solve per pair, every system, columns 0..{plain_columns - 1} "
               "timed" + ("" if plain_columns == 16 else
                          f"; x {16 // plain_columns} for the other columns (same matrices, "
                          "i.i.d. right-hand sides)")}
    out["speedup_fp64_vs_plain"] = round(all_ms / out["fp64"]["ms"], 1)
    out["speedup_fp32_refined_vs_plain"] = round(all_ms / out["fp32_inner_fp64_refined"]["ms"], 1)
    out["speedup_icc0_vs_plain"] = round(all_ms / out["fp64_icc0"]["ms"], 1)
    return out


def form_batched_sharded(torch, rank, world, pg):
    """The batched form's 512 systems x 16 right-hand sides split over the
    ranks by nnz * nrhs (batch.shard_systems): each rank solves its shard on
    its own GPU with no collective; x, its and reason are gathered on rank 0
    over gloo afterwards.  Timed: the shard solves, max over ranks."""
    from mojopetsc4py import gallery
    from mojopetsc4py.batch import sharded_solve

    systems = gallery.rgg_batch(BATCH_SYSTEMS, seed=11)
    n = sum(len(ip) - 1 for ip, _, _ in systems)
    B = np.random.default_rng(12).normal(size=(n, 16))
    t0 = time.perf_counter()
    solver, X, info = sharded_solve(systems, B, rank, world, lambda o: gather_to_root(pg, o),
                                    nrhs=16, pc="jacobi", precision="fp32", rtol=1e-8)
    setup_s = time.perf_counter() - t0
    ms = 0.0
    if solver is not None:
        Bd = torch.as_tensor(solver_rhs(solver, systems, B, rank, world), device="cuda")
        Xd = torch.empty_like(Bd)
        barrier(pg)
        ms = _sync_ms(torch, lambda: solver.solve(Bd, pc="jacobi", precision="fp32",
                                                   rtol=1e-8, out=Xd), 2)
    else:
        barrier(pg)
    ms = max_over_ranks(pg, ms)
    if rank != 0:
        return None
    return {"config": "512 RGG Laplacians x 16 RHS, CG + Jacobi, FP32 inner / FP64 refined, "
                      "rtol 1e-8, systems split over ranks by nnz * nrhs",
            "ranks": world, "max_rank_solve_ms": round(ms, 2),
            "setup_and_first_solve_s": round(setup_s, 1),
            "converged_pairs": int((info["reason"] > 0).sum()),
            "pairs": int(info["reason"].size),
            "max_true_rel_residual": float(info["relres"].max()),
            "max_its": int(info["its"].max())}


def solver_rhs(solver, systems, B, rank, world):
    """This rank's right-hand-side rows, in its shard's system order."""
    from mojopetsc4py.batch import shard_systems

    costs = [int(ip[-1]) * 16 for ip, _, _ in systems]
    mine = shard_systems(costs, world)[rank]
    offs = np.concatenate([[0], np.cumsum([len(ip) - 1 for ip, _, _ in systems])])
    return np.concatenate([B[offs[s]:offs[s + 1]] for s in mine])


def form_mixed(torch, PETSc):
    """3-D upwind convection-diffusion 96^3 (cell Peclet 10): plain FP64
    GMRES(30) + ILU(0) against FP32 inner FGMRES(30) + ILU(0) in FP64
    refinement, both held to the true FP64 residual (target 1e-10)."""
    from mojopetsc4py import gallery
    from mojopetsc4py.mixed import MixedSolver

    ip, ix, v = gallery.convection_diffusion_3d(96)
    n = len(ip) - 1
    b = np.random.default_rng(7).uniform(-1.0, 1.0, n)
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    bv = PETSc.Vec().createWithArray(b)
    out = {"config": "3-D upwind convection-diffusion 96^3, v = (1, 0.5, 0.25), cell Peclet 10, "
                     "b U[-1,1] seed 7; target ||b - A x|| <= 1e-10 ||b||",
           "n": n, "nnz": int(ip[-1])}

    def true_rel(x):
        return float(np.linalg.norm(b - _csr_matvec(ip, ix, v, x)) / np.linalg.norm(b))

    ksp = build_solver(PETSc, A, "gmres", "ilu")
    ksp.setTolerances(rtol=1e-10, atol=1e-50, divtol=1e30, max_it=MAX_IT)
    xv = PETSc.Vec().createSeq(n)
    ksp.solve(bv, xv)
    ms = _sync_ms(torch, lambda: ksp.solve(bv, xv), 1)
    out["plain_fp64_gmres30_ilu0"] = {"ms": round(ms, 2), "its": ksp.getIterationNumber(),
                                      "reason": ksp.getConvergedReason(),
                                      "true_rel_residual": true_rel(xv.getArray())}
    solver = MixedSolver(A)
    for key, sweeps in (("mixed_fp32_fgmres30_ilu0_jacobi4", 4),
                        ("mixed_fp32_fgmres30_ilu0_jacobi6", 6),
                        ("mixed_fp32_fgmres30_ilu0_exact", 0)):
        xm = PETSc.Vec().createSeq(n)
        solver.solve(bv, xm, rtol=1e-10, tri_sweeps=sweeps)
        info = {}

        def run():
            info.update(solver.solve(bv, xm, rtol=1e-10, tri_sweeps=sweeps))

        ms = _sync_ms(torch, run, 2)
        out[key] = {"ms": round(ms, 2), "passes": info["passes"],
                    "inner_its": info["inner_its"], "converged": info["converged"],
                    "true_rel_residual": true_rel(xm.getArray())}
    p = out["plain_fp64_gmres30_ilu0"]["ms"]
    out["speedup_vs_plain"] = {k: round(p / out[k]["ms"], 2) for k in out
                               if k.startswith("mixed_")}
    return out


def form_adjoint(torch, PETSc):
    """Gradient of ||u - u_obs||^2 through A(kappa) u = b, 2-D advection-
    diffusion 256^2 (Peclet 2), GMRES(30) + ILU(0) to rtol 1e-10: forward and
    adjoint solve times against the plain forward solve."""
    from mojopetsc4py import gallery
    from mojopetsc4py.adjoint import SparseSystem, sparse_solve

    k = 256
    rng = np.random.default_rng(13)
    kappa = np.exp(gallery.gaussian_random_field(k, rng, corr=16.0))
    ip, ix, v = gallery.advection_diffusion_2d(kappa, peclet=2.0)
    kappa_obs = kappa * np.exp(0.1 * gallery.gaussian_random_field(k, rng, corr=16.0))
    _, _, v_obs = gallery.advection_diffusion_2d(kappa_obs, peclet=2.0)
    n = k * k
    sysm = SparseSystem(ip, ix, ksp_type="gmres", pc_type="ilu", rtol=1e-10)
    obs = SparseSystem(ip, ix, ksp_type="gmres", pc_type="ilu", rtol=1e-12)
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    obs.set_values(torch.tensor(v_obs, device="cuda"))
    u_obs = obs.solve(b)
    vals = torch.tensor(v, device="cuda", requires_grad=True)
    rows = np.repeat(np.arange(n), np.diff(ip))
    bh = b.cpu().numpy()

    def measure(system):
        """Times and FP64 residuals of one system's forward and adjoint solves."""
        def forward():
            return sparse_solve(vals, b, system)

        def both():
            vals.grad = None
            u = forward()
            ((u - u_obs) ** 2).sum().backward()

        both()  # set-up, capture and warm-up of both solvers
        fwd_ms = _sync_ms(torch, forward, 3)
        tot_ms = _sync_ms(torch, both, 3)
        grad = vals.grad.detach().cpu().numpy()
        # residuals ||A u - b|| / ||b|| and ||A^T lam - g|| / ||g|| in FP64 on the host
        u = forward()
        uh = u.detach().cpu().numpy()
        fwd_res = float(np.linalg.norm(_csr_matvec(ip, ix, v, uh) - bh) / np.linalg.norm(bh))
        g = 2 * (u - u_obs)
        lam = system.solve_transpose(g).cpu().numpy()
        atl = np.bincount(ix, weights=v * lam[rows], minlength=n)
        gh = g.detach().cpu().numpy()
        adj_res = float(np.linalg.norm(atl - gh) / np.linalg.norm(gh))
        fs, ad = system.forward_solver, system.adjoint_solver
        out = {"forward_ms": round(fwd_ms, 2),
               "forward_plus_gradient_ms": round(tot_ms, 2),
               "gradient_over_forward": round(tot_ms / fwd_ms, 2),
               "forward_its": fs.its, "adjoint_its": ad.its,
               "forward_true_rel_residual": fwd_res,
               "adjoint_true_rel_residual": adj_res}
        if system.precision == "mixed":
            out["forward_passes"], out["adjoint_passes"] = fs.passes, ad.passes
        return out, grad

    plain, g64 = measure(sysm)
    mixed_sys = SparseSystem(ip, ix, rtol=1e-10, precision="mixed")
    mixed, gmx = measure(mixed_sys)
    mixed["gradient_rel_diff_vs_fp64"] = float(np.linalg.norm(gmx - g64) / np.linalg.norm(g64))
    return {"config": "2-D advection-diffusion 256^2, kappa = exp(GRF, corr 16 cells), "
                      "Peclet 2, upwind; loss ||u - u_obs||^2; forward and adjoint solves to "
                      "rtol 1e-10",
            "n": n, "nnz": int(ip[-1]),
            "plain_fp64_gmres30_ilu0": plain,
            "mixed_fp32_fgmres30_ilu0_refined": mixed,
            "speedup_mixed_gradient_vs_plain_gradient": round(
                plain["forward_plus_gradient_ms"] / mixed["forward_plus_gradient_ms"], 2),
            "speedup_mixed_gradient_vs_plain_forward": round(
                plain["forward_ms"] / mixed["forward_plus_gradient_ms"], 2),
            "finite_difference_equivalent_ms": round(2 * int(ip[-1]) * plain["forward_ms"], 0)}


def vec_kernels(torch, n, seed=0):
    """The Vec kernels of the bandwidth sweep on vectors of n doubles:
    (vectors, [(name, algorithmic bytes and FP64 operations per element, one
    launch through the C ABI)]); op codes as in gp_vec_map /
    gp_vec_reduce_static.  The vectors must outlive the launches."""
    import ctypes

    from mojopetsc4py import _device as dev
    from mojopetsc4py._lib import check, lib

    L, st = lib(), dev.stream_ptr()
    g = torch.Generator(device="cuda").manual_seed(seed)
    x, w, y, u, z = (torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
                     for _ in range(5))
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    X, W, Y, O = x.data_ptr(), w.data_ptr(), y.data_ptr(), out.data_ptr()
    alphas = (ctypes.c_double * 4)(0.5, -0.25, 0.125, -0.0625)
    xs = (ctypes.c_void_p * 4)(X, W, u.data_ptr(), z.data_ptr())

    def vmap(op, yp, xp=0, wp=0, a=0.5, b=0.25, c=0.125):
        return lambda: check(L.gp_vec_map(op, n, yp, xp, wp, a, b, c, st))

    def red(op, xp, yp=0):
        return lambda: check(L.gp_vec_reduce_static(op, n, xp, yp, O, st))

    kernels = [("copy", 16, 0, vmap(0, Y, X)), ("set", 8, 0, vmap(1, Y)),
               ("scale", 16, 1, vmap(2, Y, a=0.999)), ("axpy", 24, 1, vmap(4, Y, X)),
               ("aypx", 24, 1, vmap(5, Y, X)), ("axpby", 24, 2, vmap(6, Y, X)),
               ("axpbypcz", 32, 3, vmap(7, Y, X, W)), ("waxpy", 24, 1, vmap(8, Y, X, W)),
               ("pointwiseMult", 24, 1, vmap(9, Y, X, W)),
               ("maxpy4", 48, 4, lambda: check(L.gp_vec_maxpy(n, Y, 4, alphas, xs, st))),
               ("dot", 16, 1, red(0, X, W)), ("norm2", 8, 1, red(1, X)),
               ("dotNorm2", 16, 2, red(4, X, W))]
    return (x, w, y, u, z, out, alphas, xs), kernels


def run_vec_only(args):
    """Each Vec kernel of the sweep launched twice on vectors of 2^P doubles
    (the profiling target; no timing)."""
    import torch

    vs, kernels = vec_kernels(torch, 2**args.vec_only, seed=1)
    for name, _, _, fn in kernels:
        vs[2].copy_(vs[0])
        fn()
        fn()
    torch.cuda.synchronize()
    print(json.dumps({"vec_only": args.vec_only, "kernels": [k[0] for k in kernels]}),
          flush=True)


# GB300 FP64 issue rate, FMA counted as one operation: 152 SMs x 4
# sub-partitions x 32 lanes per 64 cycles at the 2.07 GHz maximum clock
# (1.26 TFLOP/s counting an FMA as two, the published FP64 figure)
FP64_OPS_PER_S = 152 * 4 * 32 / 64 * 2.07e9
L2_BYTES = 129e6


def form_bandwidth(torch, PETSc):
    """Standalone kernel sweep: the Vec kernels at n = 2^20 ... 2^26 and the
    FP64 SpMV, its transpose and the Jacobi apply on 7-point grids 64^3,
    128^3 and 160^3.

    cold    each repetition reads a 512 MB buffer first, so L2 holds clean
            lines of another buffer when the kernel starts (the read also
            covers the host's launch of the kernel), then times ONE launch
            between two CUDA events; median of the repetitions.  Vectors of
            2^20 doubles (8 MB) sit in L2 once read, so their writes need not
            reach HBM inside the timed launch: small sizes measure launch
            latency as much as bandwidth.
    stream  (launches that move more than L2 holds) the mean of 8
            back-to-back launches after one untimed launch.

    GB/s = algorithmic bytes / time.  Each kernel also has an FP64 floor, its
    FP64 operations / FP64_OPS_PER_S: on GB300 a kernel with fewer than
    ~11 bytes per FP64 operation is bound by FP64 issue before HBM (norm2,
    dotNorm2, axpby, axpbypcz; scale and the SpMV come close).  `roof_frac` =
    max(HBM floor, FP64 floor) / stream time."""
    from mojopetsc4py import _device as dev
    from mojopetsc4py import gallery
    from mojopetsc4py._lib import check, lib

    L = lib()
    st = dev.stream_ptr()
    peak, kind = peaks()
    flush = torch.ones(64 * 2**20, dtype=torch.float64, device="cuda")
    fout = torch.empty((), dtype=torch.float64, device="cuda")
    reps, burst = 15, 8

    def event():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    def timed(fn, nbytes):
        fn()
        ev = []
        for _ in range(reps):
            torch.sum(flush, dim=0, out=fout)
            e0 = event()
            fn()
            ev.append((e0, event()))
        stream = None
        if nbytes > L2_BYTES:
            fn()
            e0 = event()
            for _ in range(burst):
                fn()
            stream = (e0, event())
        torch.cuda.synchronize()
        cold = float(np.median([a.elapsed_time(b) for a, b in ev])) * 1e-3
        return cold, (stream[0].elapsed_time(stream[1]) * 1e-3 / burst if stream else None)

    def entry(nbytes, fp64_ops, fn):
        cold, stream = timed(fn, nbytes)
        out = {"cold_gbs": round(nbytes / cold / 1e9, 1)}
        if stream:
            floor = max(nbytes / (peak * 1e9), fp64_ops / FP64_OPS_PER_S)
            out.update(stream_gbs=round(nbytes / stream / 1e9, 1),
                       stream_us=round(stream * 1e6, 2),
                       hbm_floor_us=round(nbytes / (peak * 1e9) * 1e6, 2),
                       fp64_floor_us=round(fp64_ops / FP64_OPS_PER_S * 1e6, 2),
                       roof_frac=round(floor / stream, 3))
        return out

    vec = {}
    for p in (20, 22, 24, 26):
        n = 2**p
        vs, kernels = vec_kernels(torch, n, seed=p)
        for name, per, ops, fn in kernels:
            # keep y finite and of unit size whatever the updates did to it
            vs[2].copy_(vs[0])
            vec.setdefault(name, {})[f"2^{p}"] = entry(per * n, ops * n, fn)
        del vs, kernels

    mats = {}
    for k in (64, 128, 160):
        ip, ix, v = gallery.laplacian_3d(k)
        n, nnz = len(ip) - 1, int(ip[-1])
        A = PETSc.Mat().createSeqAIJ((n, n), nnz=7)
        A.setValuesCSR(ip, ix, v)
        A.assemble()
        xv = PETSc.Vec().createWithArray(np.random.default_rng(3).normal(size=n))
        yv = PETSc.Vec().createSeq(n)
        pc = PETSc.PC().create()
        pc.setType("jacobi")
        pc.setOperators(A)
        pc.setUp()
        h, xp, yp, hp = A._device(), xv._dptr(), yv._optr(), pc._handle()
        mb = (8 + spmv_index_bytes(h)) * nnz + 4 * (n + 1) + 16 * n
        mats[f"{k}^3"] = {
            "n": n, "nnz": nnz,
            "spmv": entry(mb, nnz, lambda: check(L.gp_mat_mult(h, xp, yp, st))),
            "spmv_transpose": entry(12 * nnz + 4 * (n + 1) + 16 * n, nnz, lambda: check(
                L.gp_mat_mult_transpose(h, xp, yp, st))),
            "jacobi_apply": entry(24 * n, n, lambda: check(L.gp_pc_apply(hp, xp, yp, st)))}
        del A, xv, yv, pc
    # skewed rows: a path graph with 8 hub rows of ~100k entries (row stream;
    # in the FMA arithmetic the hubs are summed by segments of 2048 slots)
    ip, ix, v = gallery.hub_laplacian(1 << 20, 8, 100_000)
    n, nnz = len(ip) - 1, int(ip[-1])
    A = PETSc.Mat().createSeqAIJ((n, n))
    A.setValuesCSR(ip, ix, v)
    A.assemble()
    xv = PETSc.Vec().createWithArray(np.random.default_rng(3).normal(size=n))
    yv = PETSc.Vec().createSeq(n)
    h, xp, yp = A._device(), xv._dptr(), yv._optr()
    mats["hubs_2^20"] = {
        "n": n, "nnz": nnz, "longest_row": int(np.diff(ip).max()),
        "spmv": entry(12 * nnz + 4 * (n + 1) + 16 * n, nnz,
                      lambda: check(L.gp_mat_mult(h, xp, yp, st)))}
    del A, xv, yv
    return {"peak_gbs": peak, "peak_kind": f"{kind} hbm_gbs",
            "fp64_ops_per_s": FP64_OPS_PER_S,
            "timing": f"cold: one launch between CUDA events after a 512 MB read, median of "
                      f"{reps}; stream: mean of {burst} back-to-back launches (launches moving "
                      "more than L2); algorithmic bytes = 8 per vector operand and element, "
                      "SpMV (8 + column bytes) nnz + 4 (n+1) + 16 n (column bytes 2 with "
                      "16-bit offsets, 4 with 32-bit indices; A^T keeps 4), Jacobi 24 n",
            "vec": vec, "sparse": mats}


def _csr_matvec(ip, ix, v, x):
    rows = np.repeat(np.arange(len(ip) - 1), np.diff(ip))
    return np.bincount(rows, weights=v * x[ix], minlength=len(ip) - 1)


def relaunch(nproc):
    """Run this script's command line under torch.distributed.run with one
    rank per GPU (rendezvous on 127.0.0.1); returns its exit status."""
    import socket

    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           f"--nproc-per-node={nproc}", "--master-addr", "127.0.0.1", "--master-port",
           str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    global MAX_IT, K3
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline solve only")
    ap.add_argument("--grid", type=int, default=K3,
                    help="grid size k of the k^3 system (128 is the benchmark; other sizes for "
                         "profiling runs)")
    ap.add_argument("--method", choices=list(METHODS), default="cg+jacobi",
                    help="method of the timed solve (cg+jacobi is the benchmark; the others "
                         "for profiling, with --quick)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--spmv-only", action="store_true", help="SpMV launches only")
    ap.add_argument("--spmv-grid", type=int, default=K3,
                    help="grid size k of the k^3 matrix for --spmv-only")
    ap.add_argument("--spmv-hubs", action="store_true",
                    help="--spmv-only on the skewed-row operator (2^20 rows, 8 hubs of ~100k)")
    ap.add_argument("--vec-only", type=int, default=None, metavar="P",
                    help="launch each Vec kernel twice on 2^P doubles (profiling)")
    ap.add_argument("--form", choices=["mixed", "batched", "adjoint", "bandwidth"], default=None,
                    help="run one of the further forms alone (profiling)")
    ap.add_argument("--batch-systems", type=int, default=512,
                    help="systems in the batched form (512 is the benchmark; fewer "
                         "only for profiling)")
    ap.add_argument("--plain-columns", type=int, default=1, choices=[1, 2, 4, 8, 16],
                    help="batched form: right-hand-side columns the plain single-system path "
                         "is timed on (16: every pair)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the mixed, batched and adjoint forms")
    ap.add_argument("--max-it", type=int, default=None,
                    help="cap the iterations (profiling runs only; not a bench value)")
    args = ap.parse_args()
    if args.max_it is not None:
        MAX_IT = args.max_it
    K3 = args.grid
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch this command under torchrun
        sys.exit(relaunch(args.gpus))
    world, rank, local, pg = dist_setup()
    if world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but {world} rank(s) were started")
    if args.form:
        import torch

        from mojopetsc4py import PETSc

        global BATCH_SYSTEMS
        BATCH_SYSTEMS = args.batch_systems
        fn = {"mixed": form_mixed,
              "batched": lambda t, P: form_batched(t, P, args.plain_columns),
              "adjoint": form_adjoint, "bandwidth": form_bandwidth}[args.form]
        print(json.dumps({"form": args.form, **fn(torch, PETSc)}), flush=True)
    elif args.spmv_only:
        run_spmv_only(args)
    elif args.vec_only is not None:
        run_vec_only(args)
    elif args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
