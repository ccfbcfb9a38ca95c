#!/usr/bin/env python
"""Benchmark: steady SIMPLE-C solves to the reference's 1e-6 residual on one GB300.

Workload (a "step" = one complete steady solve): the lid-driven cavity of the plain-method
workload -- unit cube of n^3 uniform hexahedra stored as unstructured cell/face/node lists, rho 1,
mu 0.01, lid velocity (1,0,0), no-slip walls, Re 100, the reference's relaxation 0.6/0.5 -- at
n = 48 (110,592 cells, 14x the 20^3 case), solved from the initial field until ResMax < 1e-6
(NSSolve's stop test, navier.cpp:141-145; 213 iterations at 20^3, about 880 at 48^3).  FP64
SIMPLE-C with the reference's Krylov tolerances: GMRES(30) rtol 1e-8 for u, v, w preconditioned
by a Jacobi-Neumann polynomial of degree CAVITY_POLY, CG rtol 1e-6 for the pressure correction
preconditioned by one aggregation-AMG cycle.  Every step starts from the same in-HBM restart
point (cycas_restart_point), so the K steps are K identical solves.

Metric: cell-iterations/s = cells x iterations to convergence / device time of the solves (CUDA
events on the solver's stream).  The working set of one solve (~60 MB) fits the 129 MB L2, so
the whole solve is L2-resident by design; no flush between steps.

The 480k-tet k-epsilon channel (the other plain-method workload) does not converge under the
reference's scheme: at the reference's relaxation 0.6/0.5 its pressure correction grows in a
period-2 mode until a Krylov solve fails (the reference's own sources, built single-rank in
oracle/refpin, diverge identically), and at 0.7/0.3 the residual settles into a limit cycle near
1.2e-4.  It stays available as --workload channel (a step = one SIMPLE iteration).

--impl reference times the CPU restatement of the reference (oracle/, bit-exact with the
reference's own sources; ILU(0), PETSc's one-rank default) on the same case, one
single-threaded replica per host core, each step one SIMPLE iteration of the same solve.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIG = {"nx": 200, "ny": 20, "nz": 20, "jitter": 0.15, "seed": 2026}
WORKLOAD = "kepsilon channel 200x20x20x6 jittered tets (480000 cells), FP64 SIMPLE-C"
METRIC = "cell-iters/s (steady SIMPLE-C, k-eps channel 480k tets)"
CAVITY_N = 48
CAVITY_MAX_STEP = 5000
RESIDUAL_STEADY = 1e-6
HEADLINE_WORKLOAD = ("lid-driven cavity %d^3 hexahedra (%d cells), Re 100, FP64 SIMPLE-C from the initial field "
                     "to ResMax < 1e-6" % (CAVITY_N, CAVITY_N ** 3))
HEADLINE_METRIC = "cell-iters/s to 1e-6 resid (steady SIMPLE-C, plain FP64, lid-driven cavity %d^3)" % CAVITY_N
# Degree of the Jacobi-Neumann preconditioner of the GMRES systems: single large cases (the
# 480k and 3.84M-tet channels) run fastest at 5 -- each degree adds one matrix product per Krylov
# iteration and saves iterations up to about there (GMRES ms per 10 iterations on the 480k
# channel: degree 2 39.8, 3 34.6, 4 32.7, 5 31.3, 6 32.9); batches of small cases (the cavity
# sample, the serving stream), whose systems converge in a few iterations anyway, at 1 to 3
# (degrees 1/2/3/5 on the 32-cavity batch: 73.5/73.8/74.1/69.3 M cell-iters/s).
GMRES_POLY = 5    # the k-epsilon channel (and its precision workload)
CAVITY_POLY = 2   # the cavity headline: measured 1826.7 ms per solve against 1896.1 ms for degree 5
BATCH_POLY = 2


def gmres_pc(opt, degree=None):
    """Sets the preconditioner of the GMRES systems (momentum, k, epsilon) of `opt` to the
    Jacobi-Neumann polynomial of the given degree (GMRES_POLY by default); the pressure
    correction keeps its own."""
    from sysu_cfd_parallel_gb300 import capi
    degree = GMRES_POLY if degree is None else degree
    pc = {1: capi.PC_POLY1, 2: capi.PC_POLY2, 3: capi.PC_POLY3, 4: capi.PC_POLY4, 5: capi.PC_POLY5}[degree]
    opt.ksp[capi.SYS_VELOCITY].pc = pc
    opt.ksp[capi.SYS_SCALAR].pc = pc
    return opt


def case_dir() -> str:
    base = os.environ.get("CYCAS_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "cycas_bench_cases"))
    d = os.path.join(base, "channel_%dx%dx%d_s%d" % (CONFIG["nx"], CONFIG["ny"], CONFIG["nz"], CONFIG["seed"]))
    return d


def make_case() -> str:
    from sysu_cfd_parallel_gb300 import meshgen
    d = case_dir()
    param = os.path.join(d, "param.in")
    done = os.path.join(d, "complete")
    if not os.path.exists(done):
        meshgen.write_case(d, "channel", nx=CONFIG["nx"], ny=CONFIG["ny"], nz=CONFIG["nz"], jitter=CONFIG["jitter"],
                           seed=CONFIG["seed"], steps=500)
        open(done, "w").close()
    return param


BATCH_SAMPLE = 32      # cavities of the batched sample (the 256-case workload is --workload batch256)
BATCH_SEED = 4


def batch_cases(count: int) -> list:
    """Lid-driven cavities drawn as in the batched workload: n^3 hexes with n uniform in
    {8..40}, node jitter 0.1h, Re log-uniform in [10, 1000] (mu = 1/Re), lid speed 1; cached
    on disk like the channel."""
    import numpy as np
    from sysu_cfd_parallel_gb300 import meshgen
    rng = np.random.default_rng(BATCH_SEED)
    ns = rng.integers(8, 41, size=count)
    res = 10.0 ** rng.uniform(1.0, 3.0, size=count)
    base = os.environ.get("CYCAS_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "cycas_bench_cases"))
    out = []
    for k in range(count):
        d = os.path.join(base, "cavity_batch_s%d_%03d_n%d" % (BATCH_SEED, k, ns[k]))
        param = os.path.join(d, "param.in")
        if not os.path.exists(os.path.join(d, "complete")):
            meshgen.write_case(d, "cavity", n=int(ns[k]), jitter=0.1, seed=1000 + k, steps=2000,
                               mu=float(1.0 / res[k]))
            open(os.path.join(d, "complete"), "w").close()
        out.append(param)
    return out


def timed_iterations(solver, steps: int, stream):
    """CUDA-event time of `steps` iterations on the solver's stream (ms)."""
    import torch
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.iterate(steps)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def measure_mixed(param, local, warmup, steps, ref_fields, fp64_ms):
    """The same workload with mixed-precision GMRES: throughput and the field error against the
    FP64 run after the same iterations."""
    import numpy as np
    import torch
    from sysu_cfd_parallel_gb300 import capi
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver
    case = Case(param)
    opt = gmres_pc(capi.default_options(pc=capi.PC_JACOBI, device=local))
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    opt.mixed = 1
    s = NavierStokesSolver(case, opt)
    stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
    if warmup > 0:
        s.iterate(warmup)
    ms = timed_iterations(s, steps, stream)
    err = {}
    for nm, ref in ref_fields.items():
        err[nm] = float(np.linalg.norm(s.get(nm) - ref) / np.linalg.norm(ref))
    s.close()
    return {"value": case.ncel * steps / (ms / 1e3), "ms_per_step": ms / steps,
            "speedup_vs_fp64": fp64_ms / ms,
            "krylov": "GMRES systems: FP32 Arnoldi cycles (inner rtol 1e-4) in FP64 iterative refinement",
            "field_rel_l2_vs_fp64": err}


def measure_output(s, stream, steps, plain_ms):
    """Result files of the headline case (Tecplot ASCII + res.sav backup): the synchronous writers'
    wall time, and the same files as an asynchronous dump started before `steps` iterations --
    the iterations' CUDA-event time with the dump in flight against `plain_ms` without it."""
    import shutil
    import tempfile
    import time
    import torch
    d = tempfile.mkdtemp(prefix="cycas_out_")
    try:
        t0 = time.perf_counter()
        s.Output2Tecplot(os.path.join(d, "res0000.dat"))
        s.WriteBackupFile(os.path.join(d, "res.sav"))
        sync_s = time.perf_counter() - t0
        nbytes = os.path.getsize(os.path.join(d, "res0000.dat")) + os.path.getsize(os.path.join(d, "res.sav"))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t0 = time.perf_counter()
        s.dump_begin(tecplot=os.path.join(d, "a.dat"), backup=os.path.join(d, "a.sav"))
        begin_ms = (time.perf_counter() - t0) * 1e3
        s.iterate(steps)
        e1.record(stream)
        e1.synchronize()
        t0 = time.perf_counter()
        s.dump_wait()
        wait_s = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"files": "tec/res0000.dat (Tecplot ASCII) + res.sav", "bytes": int(nbytes),
            "sync_write_s": sync_s, "async_begin_host_ms": begin_ms,
            "async_iterations_ms_per_step": ms / steps, "plain_ms_per_step": plain_ms / steps,
            "async_overhead_ms_per_step": (ms - plain_ms) / steps, "wait_after_iterations_s": wait_s}


def measure_batched(local, count, steps, mixed=False):
    """The batched sample against the same cases run one after another as single contexts."""
    import torch
    from sysu_cfd_parallel_gb300.solver import Batch, Case, NavierStokesSolver, batch_options
    params = batch_cases(count)
    opt = gmres_pc(batch_options(device=local), BATCH_POLY)
    opt.mixed = 1 if mixed else 0
    cases = [Case(p) for p in params]
    cells = sum(c.ncel for c in cases)
    b = Batch(cases, opt)
    stream = torch.cuda.ExternalStream(b.stream_handle(), device=local)
    b.iterate(2)
    ms_b = timed_iterations(b, steps, stream)
    # the autotuned team schedule, replayed as one CUDA graph per iteration
    grid, factor, _ = b.autotune(1)
    b.set_graph(True)
    b.iterate(1)
    ms_bg = timed_iterations(b, steps, stream)
    b.close()
    # the same batch with mixed-precision GMRES
    opt_m = gmres_pc(batch_options(device=local), BATCH_POLY)
    opt_m.mixed = 1
    bm = Batch(cases, opt_m)
    stream_m = torch.cuda.ExternalStream(bm.stream_handle(), device=local)
    bm.iterate(2)
    ms_bm = timed_iterations(bm, steps, stream_m)
    bm.close()
    ms_s = 0.0
    for c in cases:
        s = NavierStokesSolver(c, opt)
        st = torch.cuda.ExternalStream(s.stream_handle(), device=local)
        s.iterate(2)
        ms_s += timed_iterations(s, steps, st)
        s.close()
    return {"cases": count, "cells": cells, "value": cells * steps / (ms_b / 1e3), "ms_per_step": ms_b / steps,
            "one_case_at_a_time": {"value": cells * steps / (ms_s / 1e3), "ms_per_step": ms_s / steps},
            "speedup_vs_one_at_a_time": ms_s / ms_b,
            "autotuned_graph": {"value": cells * steps / (ms_bg / 1e3), "ms_per_step": ms_bg / steps,
                                "team_ctas": grid, "row_share_factor": factor},
            "batched_mixed": {"value": cells * steps / (ms_bm / 1e3), "ms_per_step": ms_bm / steps,
                              "speedup_vs_plain_fp64_one_at_a_time": ms_s / ms_bm},
            "mixed": bool(mixed),
            "workload": f"{count} cavities n~U{{8..40}}^3 hexes, jitter 0.1h, Re~logU[10,1000], FP64 SIMPLE-C"}


def cavity_case(n: int = CAVITY_N) -> str:
    """The headline cavity (n^3 uniform hexahedra, mu 0.01, lid 1, the reference's relaxation),
    cached on disk."""
    from sysu_cfd_parallel_gb300 import meshgen
    base = os.environ.get("CYCAS_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "cycas_bench_cases"))
    d = os.path.join(base, "cavity_%d" % n)
    param = os.path.join(d, "param.in")
    if not os.path.exists(os.path.join(d, "complete")):
        meshgen.write_case(d, "cavity", n=n, steps=CAVITY_MAX_STEP, residual=RESIDUAL_STEADY)
        open(os.path.join(d, "complete"), "w").close()
    return param


def headline_options(local: int, mixed: bool = False):
    from sysu_cfd_parallel_gb300 import capi
    opt = gmres_pc(capi.default_options(pc=capi.PC_JACOBI, device=local), CAVITY_POLY)
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    opt.mixed = 1 if mixed else 0
    return opt


L2_FLUSH_BYTES = 256 << 20  # twice the GB300's 129 MB L2


class L2Flush:
    """Writes a device buffer of twice the L2's size on the solver's stream before every timed
    step, so that no step starts on data the previous one left in L2 (256 MB: about 0.04 ms, inside
    the timed region).  Made and tried once before the timing; if that fails the flush is off and
    `state` says why."""

    def __init__(self, device, stream):
        import torch
        self.buf, self.state = None, "off"
        try:
            buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=device)
            with torch.cuda.stream(stream):
                buf.fill_(1)
            torch.cuda.synchronize()
            self.buf, self.state = buf, "on"
        except Exception as e:  # noqa: BLE001 -- a failed flush is reported, the timing goes on
            self.state = f"off ({type(e).__name__}: {e})"

    def __call__(self, stream):
        if self.buf is None:
            return
        import torch
        with torch.cuda.stream(stream):
            self.buf.fill_(1)


def solve_from_restart(s) -> dict:
    """One step: back to the restart point, then the steady loop to the stop test."""
    s.restore_restart_point()
    return s.solve_steady(CAVITY_MAX_STEP, RESIDUAL_STEADY)


def l2_note(flush) -> str:
    if flush.state == "on":
        return ("L2 flushed before every timed solve (a 256 MB write on the solver's stream, inside the timed "
                "region); within a solve its working set (< 129 MB) stays L2-resident across the SIMPLE "
                "iterations, as in any solve")
    return "no flush: the flush buffer failed, " + flush.state + "; the solve's working set is < 129 MB"


def timed_solves(s, steps: int, stream, flush=None):
    """CUDA-event time (ms) of `steps` solves on the solver's stream and the last solve's record;
    with `flush`, L2 is flushed on the stream before every solve (inside the timed region)."""
    import torch
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    iters, last = 0, None
    for _ in range(steps):
        if flush is not None:
            flush(stream)
        last = solve_from_restart(s)
        iters += last["iterations"]
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1), iters, last


def guarded(fn, *a, **kw):
    """Runs one optional leg of the bench line; its failure is reported in the line instead of
    ending the run."""
    t0 = time.time()
    try:
        out = fn(*a, **kw)
    except Exception as e:  # noqa: BLE001 -- any failure of a side leg is data for the line
        return {"error": f"{type(e).__name__}: {e}", "wall_s": time.time() - t0}
    if isinstance(out, dict):
        out.setdefault("wall_s", time.time() - t0)
    return out


def measure_mixed_solve(param, local, steps, ref_fields, fp64_ms, fp64_iters, level=1):
    # fp64_ms: the FP64 solve's time per step (ms); level 1: FP32 Arnoldi cycles, 2: also FP32
    # assembly (gradients, momentum rows, Rhie-Chow flux)
    """The headline solve with mixed-precision GMRES (FP32 Arnoldi cycles in FP64 iterative
    refinement) to the same stop test: time to converged against FP64 and the relative-L2 error of
    every field at convergence against the FP64 solve's."""
    import numpy as np
    import torch
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver
    case = Case(param)
    opt = headline_options(local, mixed=True)
    opt.mixed = level
    s = NavierStokesSolver(case, opt)
    s.set_graph(True)
    s.save_restart_point()
    stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
    solve_from_restart(s)
    ms, iters, last = timed_solves(s, steps, stream)
    err = {nm: float(np.linalg.norm(s.get(nm) - ref) / np.linalg.norm(ref)) for nm, ref in ref_fields.items()}
    s.close()
    return {"value": case.ncel * iters / (ms / 1e3), "ms_per_step": ms / steps,
            "iterations_to_converge": last["iterations"], "fp64_iterations_to_converge": fp64_iters,
            "time_to_converged_speedup_vs_fp64": fp64_ms / (ms / steps),
            "krylov": "GMRES systems: FP32 Arnoldi cycles (inner rtol 1e-4) in FP64 iterative refinement",
            "assembly": "FP32 gradients, momentum rows and Rhie-Chow flux" if level == 2 else "FP64",
            "field_rel_l2_vs_fp64_at_convergence": err}


def measure_output_solve(s, stream, plain_ms_per_solve):
    """Result files of the converged headline case (Tecplot ASCII + res.sav backup): the
    synchronous writers' wall time, and the same files as an asynchronous dump started before one
    more solve, whose CUDA-event time is compared with the plain solve's."""
    import shutil
    import torch
    d = tempfile.mkdtemp(prefix="cycas_out_")
    try:
        t0 = time.perf_counter()
        s.Output2Tecplot(os.path.join(d, "res0000.dat"))
        s.WriteBackupFile(os.path.join(d, "res.sav"))
        sync_s = time.perf_counter() - t0
        nbytes = os.path.getsize(os.path.join(d, "res0000.dat")) + os.path.getsize(os.path.join(d, "res.sav"))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t0 = time.perf_counter()
        s.dump_begin(tecplot=os.path.join(d, "a.dat"), backup=os.path.join(d, "a.sav"))
        begin_ms = (time.perf_counter() - t0) * 1e3
        solve_from_restart(s)
        e1.record(stream)
        e1.synchronize()
        t0 = time.perf_counter()
        s.dump_wait()
        wait_s = time.perf_counter() - t0
        ms = e0.elapsed_time(e1)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"files": "tec/res0000.dat (Tecplot ASCII) + res.sav", "bytes": int(nbytes), "sync_write_s": sync_s,
            "async_begin_host_ms": begin_ms, "solve_with_async_dump_ms": ms, "plain_solve_ms": plain_ms_per_solve,
            "async_overhead_ms": ms - plain_ms_per_solve, "wait_after_solve_s": wait_s}



def serve_requests(args):
    """Request stream of the serving workload (seeded): Poisson arrivals at args.rate per second
    for args.duration seconds; each request a cavity (n^3 hexes, n uniform in the cavity range,
    Re log-uniform in [10, 2000], lid speed 1) or, with equal probability, a jittered-tet k-eps
    channel (10m x m x m x 6 tets, m uniform in the channel range, inlet U log-uniform in
    [0.2, 5], mu 2e-5).  Meshes are shared between requests of the same size."""
    import numpy as np
    from sysu_cfd_parallel_gb300 import meshgen
    rng = np.random.default_rng(args.serve_seed)
    base = os.environ.get("CYCAS_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "cycas_bench_cases"))
    n_lo, n_hi = [int(v) for v in args.cavity_n.split(",")]
    m_lo, m_hi = [int(v) for v in args.channel_m.split(",")]
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / args.rate)
        if t > args.duration:
            break
        if rng.random() < 0.5:
            n = int(rng.integers(n_lo, n_hi + 1))
            re = 10.0 ** rng.uniform(1.0, np.log10(2000.0))
            mesh_dir = os.path.join(base, "serve_cavity_n%d" % n)
            if not os.path.exists(os.path.join(mesh_dir, "complete")):
                meshgen.write_case(mesh_dir, "cavity", n=n, steps=10)
                open(os.path.join(mesh_dir, "complete"), "w").close()
            text = meshgen.cavity_param(os.path.join(mesh_dir, "case.msh"), steps=100000, mu=1.0 / re)
        else:
            m = int(rng.integers(m_lo, m_hi + 1))
            u = 10.0 ** rng.uniform(np.log10(0.2), np.log10(5.0))
            mesh_dir = os.path.join(base, "serve_channel_m%d" % m)
            if not os.path.exists(os.path.join(mesh_dir, "complete")):
                meshgen.write_case(mesh_dir, "channel", nx=10 * m, ny=m, nz=m, steps=10)
                open(os.path.join(mesh_dir, "complete"), "w").close()
            text = meshgen.channel_param(os.path.join(mesh_dir, "case.msh"), steps=100000, u_in=u)
        pdir = os.path.join(base, "serve_req_s%d" % args.serve_seed)
        os.makedirs(pdir, exist_ok=True)
        param = os.path.join(pdir, "req%05d.in" % len(reqs))
        with open(param, "w") as f:
            f.write(text)
        reqs.append((t, param))
    return reqs


def run_transient(args):
    """Transient workload: the 480k-tet k-epsilon channel with the energy equation, the
    reference's second-order ("Dual") time scheme, dt 0.1 and at most 9 outer iterations per
    time step.  value: outer-iteration cell-iterations/s over `steps` time steps; the CPU sample
    is the oracle on the same mesh for one time step of one outer iteration."""
    import torch
    from sysu_cfd_parallel_gb300 import capi, meshgen
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    make_case()  # the headline mesh
    mesh = os.path.join(case_dir(), "case.msh")
    d = os.path.join(os.path.dirname(case_dir()), "transient_channel_200x20x20")
    os.makedirs(d, exist_ok=True)
    param = os.path.join(d, "param.in")
    with open(param, "w") as f:
        f.write(meshgen.channel_param(mesh, time=(0.1, 10.0, 10, "Dual"), energy=True, wall_t=290, t_in=300))
    case = Case(param)
    opt = gmres_pc(capi.default_options(pc=capi.PC_JACOBI, device=local))
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    s = NavierStokesSolver(case, opt)
    stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
    for _ in range(max(1, args.warmup)):
        s.time_step()
    clocks = Clocks(local)
    clocks.start()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    outer = 0
    for _ in range(args.steps):
        outer += s.time_step()["n"]
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    cpu = None
    if not args.no_cpu_baseline:
        import importlib
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        po = importlib.import_module("pyoracle")
        d1 = os.path.join(os.path.dirname(case_dir()), "transient_channel_200x20x20_cpu")
        os.makedirs(d1, exist_ok=True)
        p1 = os.path.join(d1, "param.in")
        with open(p1, "w") as f:
            f.write(meshgen.channel_param(mesh, time=(0.1, 10.0, 2, "Dual"), energy=True, wall_t=290, t_in=300))
        o = po.OracleCase(p1)
        for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
            o.set_ksp(w, po.PC_ILU0, 30)
        t0 = time.time()
        r = o.time_step()
        dt = time.time() - t0
        cpu = {"value": case.ncel * r["n"] / dt, "unit": "cell-iters/s", "cores": 1, "kind": "port",
               "sample": f"one time step ({r['n']} outer iteration) of the same case, oracle with ILU(0), "
                         f"{dt:.1f} s"}
    line = {"metric": "cell-iters/s (transient SIMPLE-C outer iterations, k-eps + energy channel 480k tets)",
            "value": case.ncel * outer / (ms / 1e3), "unit": "cell-iters/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(1, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "time_steps_per_s": args.steps / (ms / 1e3), "outer_iterations": outer,
            "config": {"workload": "kepsilon + energy channel 200x20x20x6 jittered tets (480000 cells), transient "
                                   "Dual scheme, dt 0.1, MaxOuterStep 10", "cells": case.ncel,
                       "step": "one physical time step"},
            "cpu_baseline": cpu, "clocks": clk}
    print(json.dumps(line), flush=True)
    s.close()


def run_precision(args):
    """Precision workload: the 400x40x40x6 channel (3.84M tets, seed 2027), plain FP64 against
    mixed-precision GMRES from the same initial state for the same iterations; throughput of
    both and the relative-L2 error of every field of the mixed run against the FP64 run."""
    import numpy as np
    import torch
    from sysu_cfd_parallel_gb300 import capi, meshgen
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    base = os.environ.get("CYCAS_BENCH_CACHE", os.path.join(tempfile.gettempdir(), "cycas_bench_cases"))
    d = os.path.join(base, "channel_400x40x40_s2027")
    param = os.path.join(d, "param.in")
    if not os.path.exists(os.path.join(d, "complete")):
        meshgen.write_case(d, "channel", nx=400, ny=40, nz=40, jitter=0.15, seed=2027, steps=500)
        open(os.path.join(d, "complete"), "w").close()
    out = {}
    fields = {}
    for mixed in (0, 1):
        case = Case(param)
        opt = gmres_pc(capi.default_options(pc=capi.PC_JACOBI, device=local))
        opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
        for k in range(3):  # the precision workload's outer tolerance, for both runs
            opt.ksp[k].rtol = args.outer_rtol
            opt.ksp[k].maxit = 5000
        opt.mixed = mixed
        s = NavierStokesSolver(case, opt)
        stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
        if args.warmup > 0:
            s.iterate(args.warmup)
        ms = timed_iterations(s, args.steps, stream)
        fields[mixed] = {nm: s.get(nm) for nm in ("U", "V", "W", "P", "TE", "ED")}
        out["mixed" if mixed else "fp64"] = {"value": case.ncel * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps}
        s.close()
    err = {nm: float(np.linalg.norm(fields[1][nm] - fields[0][nm]) / np.linalg.norm(fields[0][nm]))
           for nm in fields[0]}
    line = {"metric": "cell-iters/s (steady SIMPLE-C, k-eps channel 3.84M tets)", "unit": "cell-iters/s",
            "higher_is_better": True, "value": out["mixed"]["value"], "fp64": out["fp64"],
            "mixed": out["mixed"], "speedup_mixed_vs_fp64": out["mixed"]["value"] / out["fp64"]["value"],
            "field_rel_l2_mixed_vs_fp64": err, "steps": args.steps, "warmup": args.warmup, "n_gpus": 1,
            "dtype": "mixed", "data": "synthetic",
            "config": {"workload": "kepsilon channel 400x40x40x6 jittered tets (3840000 cells), seed 2027",
                       "krylov": "GMRES systems: FP32 Arnoldi cycles (inner rtol 1e-4) in FP64 iterative "
                                 "refinement; CG + FP32 AMG cycle (p'); every system to the outer rtol "
                                 "in both runs", "outer_rtol": args.outer_rtol}}
    print(json.dumps(line), flush=True)


def run_precision_cavity(args):
    """Precision workload, converging substitute of the 3.84M-tet channel (which does not converge
    under the reference's scheme): the lid-driven cavity at n^3 = args.side^3 solved to ResMax <
    1e-6 three times from the same initial field -- FP64, mixed level 1 (FP32 Arnoldi cycles in
    FP64 iterative refinement), mixed level 2 (also FP32 gradients, momentum rows and Rhie-Chow
    flux) -- every Krylov system to the configured outer rtol; time to converged of each and the
    relative-L2 error of every field at convergence against the FP64 run."""
    import numpy as np
    import torch
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    param = cavity_case(args.side)
    runs, fields = {}, {}
    for level in (0, 1, 2):
        case = Case(param)
        opt = headline_options(local, mixed=level > 0)
        opt.mixed = level
        for k in range(3):
            opt.ksp[k].rtol = args.outer_rtol
            opt.ksp[k].maxit = 5000
        s = NavierStokesSolver(case, opt)
        s.set_graph(True)
        stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = guarded(s.solve_steady, CAVITY_MAX_STEP, RESIDUAL_STEADY)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        its = r.get("iterations") if isinstance(r, dict) else None
        fields[level] = {nm: s.get(nm) for nm in ("U", "V", "W", "P")}
        runs[level] = {"time_to_converged_s": ms / 1e3, "iterations": its,
                       "value": case.ncel * its / (ms / 1e3) if its else None,
                       "final_resmax": float(r["resmax"][-1]) if its else None, "error": r.get("error")}
        s.close()
    for level in (1, 2):
        runs[level]["field_rel_l2_vs_fp64_at_convergence"] = {
            nm: float(np.linalg.norm(fields[level][nm] - fields[0][nm]) / np.linalg.norm(fields[0][nm]))
            for nm in fields[0]}
        runs[level]["speedup_vs_fp64"] = runs[0]["time_to_converged_s"] / runs[level]["time_to_converged_s"]
    line = {"metric": "time to ResMax < 1e-6 (steady SIMPLE-C, lid-driven cavity %d^3; mixed vs FP64)" % args.side,
            "unit": "s", "higher_is_better": False, "value": runs[2]["time_to_converged_s"], "n_gpus": 1,
            "dtype": "mixed", "data": "synthetic", "fp64": runs[0], "mixed_level1": runs[1], "mixed_level2": runs[2],
            "config": {"workload": "lid-driven cavity %d^3 hexahedra (%d cells), Re 100, to ResMax < 1e-6" %
                                   (args.side, args.side ** 3),
                       "krylov": "every system to the outer rtol (GMRES: FP32 Arnoldi cycles with inner rtol 1e-4 in "
                                 "FP64 iterative refinement in the mixed runs; CG + FP32 AMG cycle for p')",
                       "outer_rtol": args.outer_rtol}}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving workload: requests submitted at their arrival times to the continuous-batching
    server; reports time-to-converged percentiles and the aggregate cell-iterations/s."""
    import numpy as np
    import torch
    from sysu_cfd_parallel_gb300.solver import Server, batch_options
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    reqs = serve_requests(args)
    opt = gmres_pc(batch_options(device=local), BATCH_POLY)
    opt.mixed = 1 if args.mixed else 0
    srv = Server(hbm_budget_gb=args.budget_gb, residual_tol=args.tol, max_iters=args.max_iters, options=opt)
    srv.set_graph(True)
    # requests keep arriving: the next batch is built while the current one iterates
    srv.set_async_rebuild(not args.sync_rebuild)
    if args.max_cells > 0:
        srv.set_max_cells(args.max_cells)
    t0 = Server.clock()
    k = 0
    steps = 0
    while True:
        now = Server.clock() - t0
        while k < len(reqs) and reqs[k][0] <= now:
            srv.submit(reqs[k][1])
            k += 1
        active, queued = srv.step()
        steps += 1
        if k >= len(reqs) and active == 0 and queued == 0:
            break
        if Server.clock() - t0 > args.duration + args.drain:
            break
        if active == 0 and queued == 0 and k < len(reqs):
            time.sleep(max(0.0, reqs[k][0] - (Server.clock() - t0)))
    wall = Server.clock() - t0
    res = list(srv.results.values())
    lat = np.array([r["t_done"] - r["t_arrival"] for r in res]) if res else np.zeros(1)
    conv = [r for r in res if r["status"] == 1]
    cell_iters = sum(r["ncel"] * r["iterations"] for r in res)
    line = {
        "metric": "time-to-converged (serving, continuous batching)", "unit": "s", "higher_is_better": False,
        "value": float(np.percentile(lat, 99)), "p50_s": float(np.percentile(lat, 50)),
        "p99_s": float(np.percentile(lat, 99)), "requests": len(reqs), "finished": len(res),
        "converged": len(conv), "server_steps": steps, "wall_s": wall,
        "cell_iters_per_s": cell_iters / wall, "n_gpus": 1, "dtype": "f64" if not args.mixed else "mixed",
        "data": "synthetic", "loop": srv.stats(),
        "active_at_end": int(active), "queued_at_end": int(queued), "submitted": int(k),
        "config": {"workload": f"Poisson {args.rate}/s for {args.duration}s; cavities n={args.cavity_n}, "
                               f"channels m={args.channel_m}; tol {args.tol}; cap {args.max_iters} iterations; "
                               f"budget {args.budget_gb} GB; active-cell cap {args.max_cells:g}; "
                               f"drain {args.drain}s",
                   "mixed": bool(args.mixed), "batch_rebuilds": "in line" if args.sync_rebuild else "worker thread"},
    }
    print(json.dumps(line), flush=True)
    srv.close()


# ---------------------------------------------------------------- clocks
class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.device = device
        self.p = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- roofline bookkeeping
def vcycle_bytes(levels):
    """Algorithmic bytes of one AMG cycle: one pass over every level (the second cycle that
    large cases run on their shared-memory levels reads no global memory).  Per level with a
    coarser one (n rows, nnz
    entries, nc coarse rows): pre-smoothing + residual 12 nnz + 36 n, restriction 12 n + 12 nc,
    prolongation + post-smoothing 12 nnz + 40 n + 8 nc; coarsest level: dense inverse
    8 nc^2 + 16 nc."""
    rows, nnz = levels
    if len(rows) == 0:
        return 0
    b = 0
    for l in range(len(rows) - 1):
        n, z, nc = int(rows[l]), int(nnz[l]), int(rows[l + 1])
        b += 24 * z + 88 * n + 20 * nc
    nc = int(rows[-1])
    return b + 8 * nc * nc + 16 * nc


def krylov_bytes(its_row, turb, n, nnz, restart=30, levels=None, poly=0):
    """Algorithmic bytes of each Krylov launch of one iteration (solve slots in call order).

    CG iteration: reads A (12 nnz + 4 (n+1)), p, z, r, w, x, D^-1 (48 n); writes p, w, x, r, z
    (40 n); with the AMG preconditioner one cycle (vcycle_bytes) replaces D^-1.
    GMRES Arnoldi step j: SpMV + Jacobi (12 nnz + 4 (n+1) + 24 n), CGS dots (8 n (j+2)) and update
    (8 n (j+1) + 16 n); per restart cycle: initial residual (12 nnz + 4 (n+1) + 40 n) and the
    solution update (8 n (m_used + 2)).  A Jacobi-Neumann preconditioner of degree `poly` adds
    per application `poly` stages (SpMV 12 nnz + 4 (n+1), z, own row, D^-1, write: 32 n) to every
    Arnoldi step and restart residual, and |M^-1 b| once per solve (D^-1 b 24 n, its stages, the
    norm 8 n).
    """
    spmv = 12 * nnz + 4 * (n + 1)
    stage = spmv + 32 * n
    vc = vcycle_bytes(levels) if levels is not None else 0
    kinds = ["gmres", "gmres", "gmres", "cg"] + (["gmres", "gmres"] if turb else [])
    out = []
    for slot, kind in enumerate(kinds):
        its = int(its_row[slot])
        if its < 0:
            continue
        if kind == "cg":
            b = (spmv + 40 * n + vc) + its * (spmv + 88 * n + vc)
        else:
            b = (24 * n + poly * stage + 8 * n) if poly else 0
            left = its
            while True:
                m = min(left, restart)
                b += spmv + 40 * n + poly * stage
                for j in range(m):
                    b += spmv + 24 * n + poly * stage + 8 * n * (j + 2) + 8 * n * (j + 1) + 16 * n
                b += 8 * n * (m + 2)
                left -= m
                if left <= 0:
                    break
        out.append((kind, slot, its, b))
    return out


def krylov_fp64_flops(its_row, turb, n, nnz, restart=30, poly=0):
    """FP64 floating-point operations of each GMRES launch of one iteration (FP64 path): per
    Arnoldi step j the SpMV (2 nnz), the Jacobi and basis scaling (2 n), the Gram-Schmidt dots and
    update (4 n (j+1)) and the norm (2 n); per restart cycle the residual (2 nnz + 4 n) and the
    solution update (2 n m_used).  A Jacobi-Neumann preconditioner of degree `poly` adds
    2 nnz + 3 n per stage to every step and restart, and its application to D^-1 b once per
    solve.  CG slots are left out (their AMG cycle is FP32)."""
    stage = 2 * nnz + 3 * n
    kinds = ["gmres", "gmres", "gmres", "cg"] + (["gmres", "gmres"] if turb else [])
    out = []
    for slot, kind in enumerate(kinds):
        its = int(its_row[slot])
        if its < 0 or kind == "cg":
            continue
        f, left = (n + poly * stage + 2 * n) if poly else 0, its
        while True:
            m = min(left, restart)
            f += 2 * nnz + 4 * n + poly * stage
            for j in range(m):
                f += 2 * nnz + 2 * n + poly * stage + 4 * n * (j + 1) + 2 * n
            f += 2 * n * m
            left -= m
            if left <= 0:
                break
        out.append((slot, f))
    return out


def measure_fp_rates():
    """FP64 / FP32 FMA throughput of this GPU in TFLOP/s, from the bench-only probe library
    (csrc/rate_probe.cu, built beside libcycasgpu.so but not part of it)."""
    import ctypes as C
    from sysu_cfd_parallel_gb300 import build as b
    lib = C.CDLL(b.PROBE_LIB)
    lib.cycas_measure_fp_rates.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    x, y = C.c_double(), C.c_double()
    rc = lib.cycas_measure_fp_rates(C.byref(x), C.byref(y))
    if rc != 0:
        raise RuntimeError("FMA-rate probe failed (%d)" % rc)
    return x.value, y.value


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------- arms
def reduce_max(x: float, device="cpu") -> float:
    """Max of a per-rank float over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cells: int, steps: int, world: int, ms: float) -> float:
    """Cell-iterations per second of all ranks: every rank advances its own replica of the case
    by `steps` iterations; `ms` is the slowest rank's time."""
    return cells * steps * world / (ms / 1e3)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def cpu_sample(param: str, iters: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    t0 = time.time()
    o = po.OracleCase(param)
    setup = time.time() - t0
    t0 = time.time()
    o.iterate(iters)
    dt = time.time() - t0
    n = o.ncel
    o.close()
    return n * iters / dt, dt, setup, n


def _ref_replica(param, warmup, steps, barrier, q):
    """One replica of the CPU restatement (spawned process): warm up, wait for the others,
    time `steps` SIMPLE iterations."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    o = po.OracleCase(param)
    if warmup > 0:
        o.iterate(warmup)
    barrier.wait()
    t0 = time.perf_counter()
    o.iterate(steps)
    q.put((o.ncel, time.perf_counter() - t0))
    o.close()


def host_replicas(per_replica_gb=0.8):
    """Replicas of the CPU path that fit the host: one per usable core, capped so that their
    resident memory stays within half of MemAvailable."""
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count() or 1
    avail_gb = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail_gb = int(line.split()[1]) / 2**20
    except OSError:
        pass
    cap = cores if avail_gb is None else max(1, int(0.5 * avail_gb / per_replica_gb))
    return max(1, min(cores, cap)), cores


def run_reference(args):
    """The reference's CPU path on the host: the oracle restatement (bit-exact with the reference's
    own sources, which need MPI + PETSc + METIS + CGNS and do not build on the GPU host), one
    single-threaded replica of the workload per host core, ILU(0) preconditioning (PETSc's
    one-rank default).  A step is one SIMPLE iteration of the same solve the GPU arm runs to
    convergence (the CPU path takes minutes per solve), timed after `warmup` iterations."""
    import multiprocessing as mp
    rank, world, _ = dist_env()
    if rank != 0:
        return
    channel = args.workload == "channel"
    param = make_case() if channel else cavity_case()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    nproc, cores = host_replicas()
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nproc)
    q = ctx.Queue()
    procs = [ctx.Process(target=_ref_replica, args=(param, args.warmup, args.steps, barrier, q)) for _ in range(nproc)]
    for p in procs:
        p.start()
    res = [q.get() for _ in range(nproc)]
    for p in procs:
        p.join()
    n = res[0][0]
    dt = max(r[1] for r in res)
    value = n * args.steps * nproc / dt
    sample = (f"{nproc} concurrent single-threaded replicas of the {n}-cell case (one per host core of {cores}), "
              f"{args.steps} timed SIMPLE iterations each after {args.warmup} warm-up iterations of the same "
              f"solve; max over replicas")
    line = {
        "impl": "reference", "metric": METRIC if channel else HEADLINE_METRIC, "value": value, "unit": "cell-iters/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD if channel else HEADLINE_WORKLOAD, "cells": n, "replicas": nproc,
                   "step": "one SIMPLE iteration",
                   "solver": "oracle restatement of the reference (bit-exact with its own sources), ILU(0) "
                             "(PETSc one-rank default)"},
        "cpu_baseline": {"value": value, "unit": "cell-iters/s", "cores": nproc, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cell-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    """The headline: K steady solves of the cavity to ResMax < 1e-6 (device time), the same solve
    end to end through the C ABI with host buffers, the roofline of the dominant kernel, and
    the optional legs (mixed precision, batched sample, result files) each guarded."""
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver

    param = cavity_case()
    case = Case(param)
    s = NavierStokesSolver(case, headline_options(local))
    s.set_graph(True)  # every SIMPLE iteration replayed as one CUDA graph
    n, nnz, turb = case.ncel, case.nnz, case.turb_model == 1
    stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
    s.save_restart_point()
    # the initial state, kept on the host for the end-to-end leg (before any solve)
    state_names = ["U", "V", "W", "P", "R", "T", "VisLam", "VisTur", "RUFace", "BRo", "BU", "BV", "BW", "BPre",
                   "deltaP", "Apr", "dUdX", "dVdX", "dWdX", "dPdX"] + (["TE", "ED", "BTE", "BED"] if turb else [])
    host0 = {}
    for nm in state_names:
        t = torch.empty(s._size(nm), dtype=torch.float64, pin_memory=True)
        host0[nm] = t.numpy()
        host0[nm][:] = s.get(nm)

    flush = L2Flush(f"cuda:{local}", stream)
    for _ in range(max(0, args.warmup)):
        flush(stream)
        solve_from_restart(s)
    s.reset_profile()  # counts the launches of the timed region
    clocks = Clocks(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms, iters, last = timed_solves(s, args.steps, stream, flush)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches_timed = int(s.profile()["kernel_launches"])
    # per-system device times of the same solve, from CUDA events around every Krylov launch
    # (outside the timed region: the events need the launches issued one by one)
    prof_steps = max(1, min(args.steps, 3))
    s.set_graph(False)
    s.set_profiling(True)
    s.reset_profile()
    prof_ms, _, _ = timed_solves(s, prof_steps, stream, flush)
    prof = s.profile()
    s.set_profiling(False)
    s.set_graph(True)
    ms = reduce_max(ms, device="cuda")
    value = n * iters * world / (ms / 1e3)
    its_per_solve = last["iterations"]
    fields_out = ["U", "V", "W", "P"] + (["TE", "ED"] if turb else [])
    ref_fields = {nm: s.get(nm) for nm in fields_out}

    # roofline of the dominant Krylov system over the timed solves (every solve is the same)
    levels = s.amg_levels()
    per_sys_bytes = {"cg": 0.0, "gmres_vel": 0.0, "gmres_scalar": 0.0}
    per_sys_launch = {"cg": 0, "gmres_vel": 0, "gmres_scalar": 0}
    for row in last["ksp_its"]:
        for kind, slot, its, b in krylov_bytes(row, turb, n, nnz, levels=levels, poly=CAVITY_POLY):
            key = "cg" if kind == "cg" else ("gmres_vel" if slot < 3 else "gmres_scalar")
            per_sys_bytes[key] += b * prof_steps
            per_sys_launch[key] += prof_steps
    sys_ms = {"gmres_vel": prof["krylov_ms"][0], "cg": prof["krylov_ms"][1], "gmres_scalar": prof["krylov_ms"][2]}
    dom = max(sys_ms, key=lambda k: sys_ms[k])
    peak, peak_kind = measured_peak()
    launches = max(1, per_sys_launch[dom])
    achieved = (per_sys_bytes[dom] / launches) / (sys_ms[dom] / launches / 1e3) / 1e9 if sys_ms[dom] > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        try:
            t = json.load(open(tpath)).get("cavity_" + dom)
            if t:
                traffic = t["bytes_per_launch"]
        except Exception:
            traffic = None

    # end to end through the C ABI: every step uploads the initial state from pinned host
    # buffers, solves to the stop test and reads the converged fields back
    from sysu_cfd_parallel_gb300 import capi  # noqa: F401  (the ctypes layer the calls go through)
    out_names = ["U", "V", "W", "P", "RUFace"] + (["TE", "ED", "VisTur"] if turb else [])
    host_out = {}
    for nm in out_names:
        t = torch.empty(s._size(nm), dtype=torch.float64, pin_memory=True)
        host_out[nm] = t.numpy()
    h2d = sum(a.nbytes for a in host0.values())
    d2h = sum(a.nbytes for a in host_out.values()) + 8 * 10 * CAVITY_MAX_STEP
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    e2e_iters = 0
    for _ in range(e2e_steps):
        flush(stream)
        s.set_fields(host0)
        r = s.solve_steady(CAVITY_MAX_STEP, RESIDUAL_STEADY)
        e2e_iters += r["iterations"]
        s.get_fields(host_out)
    f1.record(stream)
    f1.synchronize()
    e2e_ms = reduce_max(f0.elapsed_time(f1), device="cuda")
    e2e_value = n * e2e_iters * world / (e2e_ms / 1e3)
    e2e_match = bool(e2e_iters == e2e_steps * its_per_solve)

    mixed = batched = output = None
    if not args.no_variants:
        output = guarded(measure_output_solve, s, stream, ms / args.steps)
        mixed = guarded(measure_mixed_solve, param, local, max(1, min(args.steps, 3)), ref_fields, ms / args.steps,
                        its_per_solve)
        if isinstance(mixed, dict) and "error" not in mixed:
            mixed["fp32_assembly"] = guarded(measure_mixed_solve, param, local, max(1, min(args.steps, 3)),
                                             ref_fields, ms / args.steps, its_per_solve, 2)
        batched = guarded(measure_batched, local, BATCH_SAMPLE, 10)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = guarded(cpu_baseline_leg, param, args.cpu_iters)

    if rank == 0:
        line = {
            "metric": HEADLINE_METRIC, "value": value, "unit": "cell-iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": HEADLINE_WORKLOAD, "step": "one steady solve from the initial field to "
                                                              "ResMax < 1e-6 (restart point restored first)",
                       "cells": n, "faces": case.nfac, "nnz": nnz, "iterations_to_converge": its_per_solve,
                       "final_resmax": float(last["resmax"][-1]),
                       "parallelism": f"replicas{world}", "l2": l2_note(flush),
                       "krylov": "GMRES(30) rtol 1e-8 with the Jacobi-Neumann polynomial preconditioner of degree %d "
                                 "(u,v,w), CG rtol 1e-6 + AMG cycle (p'), the reference's tolerances" % CAVITY_POLY,
                       "krylov_its_first_iteration": [int(x) for x in last["ksp_its"][0]],
                       "krylov_its_last_iteration": [int(x) for x in last["ksp_its"][-1]],
                       "amg_levels_rows": [int(x) for x in levels[0]]},
            "e2e": {"value": e2e_value, "unit": "cell-iters/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps, "same_iterations_as_device_run": e2e_match,
                    "path": "C ABI: cycas_set_fields (initial state from pinned host buffers) + cycas_solve_steady "
                            "+ cycas_get_fields (converged fields)"},
            "roofline": {"bound": "hbm", "kernel": {"cg": "k_cg_amg (pressure correction: CG + AMG cycle)",
                                                    "gmres_vel": "k_gmres_ms<3> (u, v, w in lockstep)",
                                                    "gmres_scalar": "k_gmres_ms<1> (k, epsilon)"}[dom],
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "share_of_step": sys_ms[dom] / prof_ms,
                         "launches": per_sys_launch[dom], "timing": "CUDA events around every launch of "
                         "the system over %d untimed solves of the same case" % prof_steps},
            "cpu_baseline": cpu,
            "mixed": mixed,
            "batched": batched,
            "output": output,
            "gpu_launches": launches_timed,
            "profile": {"solves": prof_steps, "solve_ms": prof_ms / prof_steps, "krylov_ms": sys_ms,
                        "assembly_ms": prof["assembly_ms"], "krylov_iters": prof["krylov_iters"]},
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline_leg(param: str, iters: int) -> dict:
    v, dt, setup, _ = cpu_sample(param, iters)
    return {"value": v, "unit": "cell-iters/s", "cores": 1, "kind": "port",
            "sample": f"the first {iters} SIMPLE iterations of the same solve, oracle (bit-exact with the "
                      f"reference's own sources) with ILU(0), PETSc's one-rank default, {dt:.1f} s after "
                      f"{setup:.1f} s setup"}


def run_channel(args):
    """The k-epsilon channel workload: a step = one SIMPLE iteration of the 480k-tet channel (which
    does not converge under the reference's scheme; see the module docstring)."""
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from sysu_cfd_parallel_gb300 import capi
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver

    fp64_peak, fp32_peak = measure_fp_rates()
    param = make_case()
    case = Case(param)
    opt = gmres_pc(capi.default_options(pc=capi.PC_JACOBI, device=local))
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    s = NavierStokesSolver(case, opt)
    n, nnz, turb = case.ncel, case.nnz, case.turb_model == 1
    stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)

    if args.warmup > 0:
        s.iterate(args.warmup)
    s.set_profiling(True)
    s.reset_profile()
    clocks = Clocks(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    hist = s.iterate(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    prof = s.profile()
    ref_fields = {nm: s.get(nm) for nm in (["U", "V", "W", "P"] + (["TE", "ED"] if turb else []))}
    ms = reduce_max(ms, device="cuda")
    value = whole_job_rate(n, args.steps, world, ms)

    # roofline of the dominant Krylov system
    levels = s.amg_levels()
    per_sys_bytes = {"cg": 0.0, "gmres_vel": 0.0, "gmres_scalar": 0.0}
    per_sys_launch = {"cg": 0, "gmres_vel": 0, "gmres_scalar": 0}
    for row in hist["ksp_its"]:
        for kind, slot, its, b in krylov_bytes(row, turb, n, nnz, levels=levels, poly=GMRES_POLY):
            key = "cg" if kind == "cg" else ("gmres_vel" if slot < 3 else "gmres_scalar")
            per_sys_bytes[key] += b
            per_sys_launch[key] += 1
    sys_ms = {"gmres_vel": prof["krylov_ms"][0], "cg": prof["krylov_ms"][1], "gmres_scalar": prof["krylov_ms"][2]}
    dom = max(sys_ms, key=lambda k: sys_ms[k])
    peak, peak_kind = measured_peak()
    launches = max(1, per_sys_launch[dom])
    achieved = (per_sys_bytes[dom] / launches) / (sys_ms[dom] / launches / 1e3) / 1e9 if sys_ms[dom] > 0 else 0.0
    # FP64 roofline of the GMRES system with the larger share (the CG's AMG cycle is FP32)
    gdom = "gmres_vel" if sys_ms["gmres_vel"] >= sys_ms["gmres_scalar"] else "gmres_scalar"
    flops = sum(f for row in hist["ksp_its"] for slot, f in krylov_fp64_flops(row, turb, n, nnz, poly=GMRES_POLY)
                if (slot < 3) == (gdom == "gmres_vel"))
    ach = flops / (sys_ms[gdom] / 1e3) / 1e12 if sys_ms[gdom] > 0 else 0.0
    fp64 = {"kernel": gdom, "achieved_tflops": ach, "peak_tflops": fp64_peak, "peak_kind": "measured live",
            "frac": ach / fp64_peak if fp64_peak > 0 else None, "fp32_peak_tflops": fp32_peak}
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        # DRAM bytes of one captured launch (ncu), scaled to this run's mean Krylov iterations
        # per launch of the same system (the traffic grows with the iterations)
        try:
            t = json.load(open(tpath)).get(dom)
            if t:
                its = [x[2] for row in hist["ksp_its"]
                       for x in krylov_bytes(row, turb, n, nnz, levels=levels, poly=GMRES_POLY)
                       if {"cg": x[0] == "cg", "gmres_vel": x[0] == "gmres" and x[1] < 3,
                           "gmres_scalar": x[0] == "gmres" and x[1] >= 3}[dom]]
                traffic = t["bytes"] * (sum(its) / len(its)) / t["its"] if its else None
        except Exception:
            traffic = None

    # end to end through the C ABI: the caller's host arrays are the state (pinned buffers),
    # uploaded into and read back from every iteration (cycas_simple_iteration_io: each copy
    # overlaps the stages that do not touch its field)
    names_in = ["U", "V", "W", "P", "R", "VisLam", "VisTur", "TE", "ED", "RUFace", "BRo", "BU", "BV", "BW",
                "BTE", "BED"]
    names_out = ["U", "V", "W", "P", "VisTur", "TE", "ED", "RUFace"]
    host = {}
    for nm in set(names_in) | set(names_out):
        t = torch.empty(s._size(nm), dtype=torch.float64, pin_memory=True)
        host[nm] = t.numpy()
        host[nm][:] = s.get(nm)
    h2d = sum(host[nm].nbytes for nm in names_in)
    d2h = sum(host[nm].nbytes for nm in names_out) + 8 * 10
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    up = {nm: host[nm] for nm in names_in}
    down = {nm: host[nm] for nm in names_out}
    for _ in range(e2e_steps):
        s.simple_iteration_io(up, down)  # uploads and downloads overlap the iteration's stages
    f1.record(stream)
    f1.synchronize()
    e2e_ms = f0.elapsed_time(f1)
    e2e_ms = reduce_max(e2e_ms, device="cuda")
    e2e_value = whole_job_rate(n, e2e_steps, world, e2e_ms)

    mixed = batched = output = None
    if not args.no_variants:
        output = guarded(measure_output, s, stream, args.steps, ms)
        mixed = guarded(measure_mixed, param, local, args.warmup, args.steps, ref_fields, ms)
        batched = guarded(measure_batched, local, BATCH_SAMPLE, args.steps)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = guarded(cpu_baseline_leg, param, min(args.cpu_iters, 3))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": n, "faces": case.nfac, "nnz": nnz,
                       "parallelism": f"replicas{world}", "l2": "working set > 129 MB L2, no flush",
                       "krylov": "GMRES(30) with the Jacobi-Neumann polynomial preconditioner of degree %d "
                                 "(u,v,w,k,eps), CG+AMG cycle (p'), reference tolerances" % GMRES_POLY,
                       "krylov_its_last_step": [int(x) for x in hist["ksp_its"][-1]],
                       "amg_levels_rows": [int(x) for x in levels[0]],
                       "amg_levels_nnz": [int(x) for x in levels[1]]},
            "e2e": {"value": e2e_value, "unit": "cell-iters/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
            "roofline": {"bound": "hbm", "kernel": {"cg": "k_cg_amg (pressure correction: CG + AMG cycle)",
                                                    "gmres_vel": "k_gmres_ms<3> (u, v, w in lockstep)",
                                                    "gmres_scalar": "k_gmres_ms<1> (k, epsilon)"}[dom],
                         "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "share_of_step": sys_ms[dom] / ms},
            "fp64_roofline": fp64,
            "cpu_baseline": cpu,
            "mixed": mixed,
            "batched": batched,
            "output": output,
            "gpu_launches": int(prof["kernel_launches"]),
            "profile": {"krylov_ms": sys_ms, "assembly_ms": prof["assembly_ms"],
                        "krylov_iters": prof["krylov_iters"]},
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch256(args):
    """The batching workload as configured: 256 lid-driven cavities (n^3 hexahedra, n uniform in
    {8..40}, node jitter 0.1h, Re log-uniform in [10, 1000], lid speed 1), every one solved to a
    1e-6 residual (ResMax / cell volume sum, the cube's volume being 1).  Three legs:
      * batched: all cases submitted at once to the continuous-batching server, FP64, every
        batch iteration replayed as one CUDA graph; a case leaves the batch when it converges;
      * batched + mixed: the same with mixed-precision GMRES (FP32 Arnoldi cycles in FP64
        iterative refinement);
      * one at a time: each case alone through cycas_solve_steady, plain FP64 with the
        headline's preconditioners (the plain FP64 GPU path).
    value: cell-iterations/s of the batched + mixed leg (every case's iterations to convergence
    over the wall time from submission to the last retirement)."""
    import numpy as np
    import torch
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver, Server
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    params = batch_cases(args.batch_cases)
    ncel = [Case(p).ncel for p in params]
    cells = sum(ncel)

    def served(mixed):
        opt = gmres_pc(batch_options_local(local), BATCH_POLY)
        opt.mixed = 1 if mixed else 0
        srv = Server(hbm_budget_gb=args.budget_gb, residual_tol=args.tol, max_iters=args.max_iters, options=opt)
        srv.set_graph(True)
        srv.set_async_rebuild(args.async_rebuild)
        t0 = Server.clock()
        ids = [srv.submit(p) for p in params]
        steps = 0
        while True:
            active, queued = srv.step()
            steps += 1
            if active == 0 and queued == 0:
                break
        wall = Server.clock() - t0
        res = [srv.results[i] for i in ids]
        st = srv.stats()
        srv.close()
        its = np.array([r["iterations"] for r in res])
        conv = sum(r["status"] == 1 for r in res)
        lat = np.array([r["t_done"] - r["t_arrival"] for r in res])
        return {"wall_s": wall, "value": float(np.dot(its, ncel)) / wall, "converged": int(conv),
                "cases": len(res), "iterations": its.tolist(), "server_steps": steps,
                "time_to_converged_p50_s": float(np.percentile(lat, 50)),
                "time_to_converged_p99_s": float(np.percentile(lat, 99)), "loop": st}

    out = {"batched": guarded(served, False), "batched_mixed": guarded(served, True)}

    def alone():
        from sysu_cfd_parallel_gb300 import capi
        total_ms, its, fails = 0.0, [], 0
        for p in params:
            s = NavierStokesSolver(Case(p), headline_options(local))
            stream = torch.cuda.ExternalStream(s.stream_handle(), device=local)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            try:
                r = s.solve_steady(args.max_iters, args.tol)
                its.append(r["iterations"])
                fails += 0 if r["resmax"][-1] < args.tol else 1
            except capi.CycasError:
                its.append(-1)
                fails += 1
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            s.close()
        good = np.array([max(0, i) for i in its])
        return {"device_s": total_ms / 1e3, "value": float(np.dot(good, ncel)) / (total_ms / 1e3),
                "iterations": its, "not_converged": fails}

    if not args.no_variants:
        out["one_at_a_time_plain_fp64"] = guarded(alone)
    bm = out["batched_mixed"]
    line = {"metric": "cell-iters/s to 1e-6 resid (256 cavities, batched + mixed vs plain FP64 one at a time)",
            "value": bm.get("value"), "unit": "cell-iters/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "mixed", "data": "synthetic", "cells": cells,
            "config": {"workload": "%d cavities n~U{8..40}^3 hexahedra, jitter 0.1h, Re~logU[10,1000], each to "
                                   "1e-6; continuous-batching server, CUDA graph per batch iteration" % len(params),
                       "budget_gb": args.budget_gb, "max_iters": args.max_iters,
                       "batch_rebuilds": "worker thread" if args.async_rebuild else "in line"},
            **out}
    a = out.get("one_at_a_time_plain_fp64") or {}
    for k in ("batched", "batched_mixed"):
        if "wall_s" in out[k] and "device_s" in a:
            out[k]["speedup_vs_one_at_a_time_plain_fp64"] = a["device_s"] / out[k]["wall_s"]
    print(json.dumps(line), flush=True)


def batch_options_local(local):
    from sysu_cfd_parallel_gb300.solver import batch_options
    return batch_options(device=local)


def run_profile(args):
    """Profiling leg (for ncu and per-system timings): `--steps` SIMPLE iterations of a generated
    case after `--warmup` untimed ones, with the per-system Krylov timing of the library on; prints
    one JSON line with the Krylov iteration counts and the profile."""
    from sysu_cfd_parallel_gb300 import capi, meshgen
    from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver
    d = tempfile.mkdtemp(prefix="cycas_prof_")
    iters = args.steps + args.warmup
    if args.kind == "channel":
        kw = {"jitter": args.jitter, "seed": 2026} if args.jitter > 0 else {}
        param = meshgen.write_case(d, "channel", nx=args.nx, ny=args.ny, nz=args.nz, steps=iters, **kw)
    else:
        kw = {"jitter": args.jitter, "seed": 1000} if args.jitter > 0 else {}
        param = meshgen.write_case(d, "cavity", n=args.side, steps=iters, **kw)
    opt = capi.default_options(pc=capi.PC_JACOBI)
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG if args.pressure_pc == "amg" else capi.PC_JACOBI
    opt.mixed = 1 if args.mixed else 0
    opt.amg_omega = args.amg_omega
    opt.amg_gamma = args.amg_gamma
    gpc = {"jacobi": capi.PC_JACOBI, "poly1": capi.PC_POLY1, "poly2": capi.PC_POLY2, "poly3": capi.PC_POLY3,
           "poly4": capi.PC_POLY4, "poly5": capi.PC_POLY5}[
        args.gmres_pc or "poly%d" % (GMRES_POLY if args.kind == "channel" else CAVITY_POLY)]
    opt.ksp[capi.SYS_VELOCITY].pc = gpc
    opt.ksp[capi.SYS_SCALAR].pc = gpc
    s = NavierStokesSolver(Case(param), opt)
    if args.warmup:
        s.iterate(args.warmup)
    s.set_profiling(True)
    s.reset_profile()
    t0 = time.time()
    r = s.iterate(args.steps)
    dt = time.time() - t0
    print(json.dumps({"workload": "profile", "cells": s.case.ncel, "iters": args.steps, "seconds": dt,
                      "ksp_its": r["ksp_its"].tolist(), "profile": s.profile()}), flush=True)
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-iters", type=int, default=15)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the mixed-precision and batched lines")
    ap.add_argument("--workload", default="cavity",
                    choices=["cavity", "channel", "serve", "precision", "precision_cavity", "transient", "profile",
                             "batch256"])
    ap.add_argument("--batch-cases", type=int, default=256, help="batch256 workload: number of cavities")
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--drain", type=float, default=120.0)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--max-iters", type=int, default=3000)
    ap.add_argument("--cavity-n", default="16,64")
    ap.add_argument("--channel-m", default="10,25")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--max-cells", type=float, default=4e6,
                    help="serve workload: cap on the active requests' cells (0: HBM budget only)")
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--sync-rebuild", action="store_true",
                    help="serve workload: rebuild batches in line instead of on a worker thread")
    ap.add_argument("--async-rebuild", action="store_true",
                    help="batch256 workload: rebuild batches on a worker thread")
    ap.add_argument("--serve-seed", type=int, default=5)
    ap.add_argument("--outer-rtol", type=float, default=1e-10, help="precision workload: rtol of every system")
    # --workload profile: the generated case and its solver options
    ap.add_argument("--kind", default="cavity", choices=["channel", "cavity"])
    ap.add_argument("--nx", type=int, default=100)
    ap.add_argument("--ny", type=int, default=10)
    ap.add_argument("--nz", type=int, default=10)
    ap.add_argument("--side", type=int, default=CAVITY_N, help="cavity cells per side")
    ap.add_argument("--pressure-pc", default="amg", choices=["amg", "jacobi"])
    ap.add_argument("--gmres-pc", default=None, choices=["jacobi", "poly1", "poly2", "poly3", "poly4", "poly5"],
                    help="profile workload: GMRES preconditioner (default: the workload's bench setting)")
    ap.add_argument("--amg-omega", type=float, default=0.0, help="AMG smoother weight (0: library default)")
    ap.add_argument("--amg-gamma", type=int, default=0, help="AMG cycles at the first shared-memory level")
    ap.add_argument("--jitter", type=float, default=0.0, help="interior node jitter (fraction of h)")
    args = ap.parse_args()
    if args.workload == "profile":
        run_profile(args)
    elif args.workload == "batch256":
        run_batch256(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "precision_cavity":
        run_precision_cavity(args)
    elif args.workload == "transient":
        run_transient(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "channel":
        run_channel(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
