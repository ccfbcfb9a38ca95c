"""Full-length runs on the GPU against the reference build and the oracle.

* The plain-method cavity (20^3 hexahedra, Re 100) for its configured 200 SIMPLE iterations with
  GMRES(30) rtol 1e-8 on every system and Jacobi preconditioning, against the fixture the
  reference's own sources wrote (tests/golden/cavity20/ref_jacobi.npz): residual history to
  relative 1e-6, u, v, w, p to relative L2 1e-8, Krylov counts within one.
* The same cavity with the headline's preconditioners (Jacobi-Neumann polynomial of degree 2 for
  the momentum GMRES -- and degree 5, the channel's -- CG + aggregation AMG for the pressure
  correction) against the oracle with
  the reference's ILU(0), every system solved tightly on both sides (rtol 1e-12; 1e-10 for the
  pressure correction, whose singular pure-Neumann system ILU(0)-CG cannot take further in FP64):
  with the Krylov error made negligible the SIMPLE iterations must coincide whatever the
  preconditioner -- residual
  history to relative 1e-6, fields to 1e-8, and both cross NSSolve's stop test (ResMax < 1e-6,
  navier.cpp:141-145) at the same iteration.
* The bench's cavity (48^3 hexahedra) for its first 5 SIMPLE iterations with the headline's
  preconditioners, solved tightly (rtol 1e-12; 1e-10 for the pressure correction), against the
  fixture the reference's own sources wrote with ILU(0) and rtol 1e-10
  (tests/golden/cavity48/ref_ilu_tight.npz): residual history to relative 1e-6, the L2 norm of
  u, v, w, p to relative 1e-8 and their sums to 1e-8 of norm x sqrt(cells).  On the CPU the
  oracle's ILU(0) and Jacobi runs at these tolerances differ from the fixture by at most 1.5e-8
  (residuals), 7e-11 (norms) and 6e-11 (sums): the Krylov error of the fixture itself.
* The steady loop (cycas_solve_steady) and the in-HBM restart point on a small case: the loop
  stops where the oracle's NSSolve loop stops, and a restored restart point repeats the solve
  bit for bit.
"""
import os
import sys

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


def _cavity20(tmp_path):
    from make_ref_golden import write_cavity20
    return os.path.join(write_cavity20(str(tmp_path)), "param.in")


def test_cavity20_configured_run_matches_reference_build(tmp_path):
    g = dict(np.load(os.path.join(GOLDEN, "cavity20", "ref_jacobi.npz")))
    opt = capi.default_options(pc=capi.PC_JACOBI)
    for k in range(3):
        opt.ksp[k].type = capi.KSP_GMRES
        opt.ksp[k].rtol = 1e-8
    s = NavierStokesSolver(Case(_cavity20(tmp_path)), opt)
    r = s.iterate(200)
    res_ref = g["residual"]
    np.testing.assert_allclose(r["residual"], res_ref, rtol=1e-6, atol=1e-300)
    its_ref = g["ksp"][:, 1].astype(np.int32).reshape(200, 4)
    assert np.all(np.abs(r["ksp_its"][:, :4] - its_ref) <= 1)
    for nm in ("U", "V", "W", "P"):
        err = _rel_l2(s.get(nm), g[nm])
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"
    s.close()


def test_cavity48_first_iterations_match_reference_build(tmp_path):
    from make_ref_golden import write_cavity48
    g = dict(np.load(os.path.join(GOLDEN, "cavity48", "ref_ilu_tight.npz")))
    param = os.path.join(write_cavity48(str(tmp_path)), "param.in")
    opt = capi.default_options(pc=capi.PC_POLY2)
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    for k in range(3):
        opt.ksp[k].rtol = 1e-10 if k == capi.SYS_PRESSURE else 1e-12
        opt.ksp[k].maxit = 5000
    s = NavierStokesSolver(Case(param), opt)
    r = s.iterate(int(g["steps"]))
    np.testing.assert_allclose(r["residual"], g["residual"], rtol=1e-6, atol=1e-300)
    sq = np.sqrt(48 ** 3)
    for nm in ("U", "V", "W", "P"):
        x, nref = s.get(nm), float(g[nm + "_norm"])
        assert abs(np.linalg.norm(x) - nref) <= 1e-8 * nref, nm
        assert abs(np.sum(x) - float(g[nm + "_sum"])) <= 1e-8 * nref * sq, nm
    s.close()


@pytest.mark.parametrize("poly", [2, 5])
def test_cavity20_headline_preconditioners_match_oracle_ilu(tmp_path, poly):
    param = _cavity20(tmp_path)
    o = po.OracleCase(param)
    rtol = {po.VELOCITY: 1e-12, po.PRESSURE: 1e-10, po.SCALAR: 1e-12}
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, po.PC_ILU0, 30, rtol[w], 5000)
    opt = capi.default_options(pc={2: capi.PC_POLY2, 5: capi.PC_POLY5}[poly])
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    for k in range(3):
        opt.ksp[k].rtol = rtol[k]
        opt.ksp[k].maxit = 5000
    s = NavierStokesSolver(Case(param), opt)
    ro_res, ro_rm = [], []
    stop_o = None
    for it in range(1, 401):
        r = o.iterate(1)
        ro_res.append(r["residual"][0])
        ro_rm.append(r["resmax"][0])
        if r["resmax"][0] < 1e-6:
            stop_o = it
            break
    rg = s.solve_steady(400, 1e-6)
    assert stop_o is not None and rg["iterations"] == stop_o, (rg["iterations"], stop_o)
    np.testing.assert_allclose(rg["residual"], np.array(ro_res), rtol=1e-6, atol=1e-300)
    for nm in ("U", "V", "W", "P"):
        err = _rel_l2(s.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"
    s.close()
    o.close()


def test_solve_steady_stop_and_restart_point(cases):
    param = cases("cavity8")
    o = po.OracleCase(param)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, po.PC_JACOBI)
    s = NavierStokesSolver(Case(param), capi.default_options(pc=capi.PC_JACOBI))
    s.save_restart_point()
    tol = 1e-5
    stop_o = None
    for it in range(1, 1000):
        if o.iterate(1)["resmax"][0] < tol:
            stop_o = it
            break
    r1 = s.solve_steady(1000, tol)
    assert r1["iterations"] == stop_o
    assert r1["resmax"][-1] < tol and np.all(r1["resmax"][:-1] >= tol)
    u1 = s.get("U")
    s.restore_restart_point()
    r2 = s.solve_steady(1000, tol)
    assert r2["iterations"] == r1["iterations"]
    assert np.array_equal(r2["resmax"].view(np.int64), r1["resmax"].view(np.int64))
    assert np.array_equal(s.get("U").view(np.int64), u1.view(np.int64))
    # a cap below the crossing stops at the cap
    s.restore_restart_point()
    r3 = s.solve_steady(3, tol)
    assert r3["iterations"] == 3
    s.close()
    o.close()
