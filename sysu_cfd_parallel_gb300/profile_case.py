"""Run a few SIMPLE iterations of a generated case (for profilers such as ncu).

    python -m sysu_cfd_parallel_gb300.profile_case --kind channel --nx 100 --ny 10 --nz 10 --iters 2

prints one JSON line with the per-iteration Krylov iteration counts and timings.
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--kind", default="channel", choices=["channel", "cavity"])
    ap.add_argument("--nx", type=int, default=100)
    ap.add_argument("--ny", type=int, default=10)
    ap.add_argument("--nz", type=int, default=10)
    ap.add_argument("--n", type=int, default=20, help="cavity cells per side")
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--pressure-pc", default="amg", choices=["amg", "jacobi"])
    ap.add_argument("--mixed", action="store_true", help="FP32 Arnoldi cycles in FP64 refinement")
    ap.add_argument("--pc", default="jacobi", choices=["jacobi", "poly1", "poly2", "poly3", "poly4", "poly5"],
                    help="preconditioner of the GMRES systems (momentum, scalars)")
    ap.add_argument("--warmup", type=int, default=0, help="untimed iterations before the profiled ones")
    ap.add_argument("--amg-omega", type=float, default=0.0, help="AMG smoother weight (0: library default)")
    ap.add_argument("--amg-gamma", type=int, default=0, help="AMG cycles at the first shared-memory level")
    ap.add_argument("--jitter", type=float, default=0.0, help="interior node jitter (fraction of h)")
    args = ap.parse_args(argv)

    from . import capi, meshgen
    from .solver import Case, NavierStokesSolver

    d = tempfile.mkdtemp(prefix="cycas_prof_")
    if args.kind == "channel":
        kw = {"jitter": args.jitter, "seed": 2026} if args.jitter > 0 else {}
        param = meshgen.write_case(d, "channel", nx=args.nx, ny=args.ny, nz=args.nz, steps=args.iters + args.warmup,
                                   **kw)
    else:
        kw = {"jitter": args.jitter, "seed": 1000} if args.jitter > 0 else {}
        param = meshgen.write_case(d, "cavity", n=args.n, steps=args.iters + args.warmup, **kw)
    opt = capi.default_options(pc=capi.PC_JACOBI)
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG if args.pressure_pc == "amg" else capi.PC_JACOBI
    opt.mixed = 1 if args.mixed else 0
    opt.amg_omega = args.amg_omega
    opt.amg_gamma = args.amg_gamma
    gpc = {"jacobi": capi.PC_JACOBI, "poly1": capi.PC_POLY1, "poly2": capi.PC_POLY2, "poly3": capi.PC_POLY3,
           "poly4": capi.PC_POLY4, "poly5": capi.PC_POLY5}[args.pc]
    opt.ksp[capi.SYS_VELOCITY].pc = gpc
    opt.ksp[capi.SYS_SCALAR].pc = gpc
    s = NavierStokesSolver(Case(param), opt)
    if args.warmup:
        s.iterate(args.warmup)
    s.set_profiling(True)
    s.reset_profile()
    t0 = time.time()
    r = s.iterate(args.iters)
    dt = time.time() - t0
    print(json.dumps({"cells": s.case.ncel, "iters": args.iters, "seconds": dt,
                      "ksp_its": r["ksp_its"].tolist(), "profile": s.profile()}))
    s.close()


if __name__ == "__main__":
    main()
