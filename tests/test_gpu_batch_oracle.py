"""Batched and served cases against the CPU oracle run alone.

A batch (block-diagonal systems, one persistent launch per phase for all cases) and the
continuous-batching server must give every case the iterations the reference gives it alone.
Here the reference is the oracle: each case of a small batch, and each request of a small
served stream, is compared with the oracle solving that case by itself for the same number of
SIMPLE iterations.  The GPU runs its batch preconditioners (Jacobi-Neumann polynomial for the
GMRES systems, CG + AMG for the pressure correction), the oracle the reference's ILU(0); with
every Krylov solve taken tight on both sides (rtol 1e-12, 1e-10 for the oracle's pressure
correction, whose singular system ILU(0)-CG takes no further) the preconditioner no longer
matters and the fields agree to relative L2 1e-8.
"""
import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import Batch, Case, Server, batch_options

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


def _tight_gpu():
    o = batch_options(pc=capi.PC_POLY2)
    for k in range(3):
        o.ksp[k].rtol = 1e-12
        o.ksp[k].maxit = 5000
    return o


def _oracle_alone(param, iters):
    o = po.OracleCase(param)
    for w, rt in ((po.VELOCITY, 1e-12), (po.PRESSURE, 1e-10), (po.SCALAR, 1e-12)):
        o.set_ksp(w, po.PC_ILU0, 30, rt, 5000)
    r = o.iterate(iters)
    return o, r


def test_batched_cases_match_oracle_alone(cases):
    params = [cases(n) for n in ("cavity8", "cavity8j", "cavity4")]  # one physics class per batch
    b = Batch([Case(p) for p in params], _tight_gpu())
    rb = b.iterate(10)
    for k, p in enumerate(params):
        o, ro = _oracle_alone(p, 10)
        np.testing.assert_allclose(rb["resmax"][:, k], ro["resmax"], rtol=1e-6)
        for nm in ("U", "V", "W", "P"):
            err = _rel_l2(b.case_field(nm, k), o.get(nm))
            assert err < 1e-8, f"case {k} {nm}: relative L2 {err:.3e}"
        o.close()
    b.close()


@pytest.mark.parametrize("async_rebuild", [False, True])
def test_served_requests_match_oracle_alone(cases, async_rebuild):
    """Also with batches rebuilt on a worker thread: the late arrival's batch is built while the
    first two requests keep iterating, and their state moves over at the switch."""
    names = ["cavity4", "cavity8", "channel_tiny"]
    params = {n: cases(n) for n in names}
    srv = Server(hbm_budget_gb=100.0, residual_tol=1e-5, max_iters=12, keep_fields=True, options=_tight_gpu())
    srv.set_async_rebuild(async_rebuild)
    ids = {n: srv.submit(params[n]) for n in names[:2]}
    for step in range(100):
        if step == 2:  # a later arrival joins the running server
            ids[names[2]] = srv.submit(params[names[2]])
        active, queued = srv.step()
        if step > 2 and active == 0 and queued == 0:
            break
    assert len(srv.results) == len(names)
    for n in names:
        r = srv.results[ids[n]]
        case = Case(params[n])
        o, _ = _oracle_alone(params[n], r["iterations"])
        fields = ["U", "V", "W", "P"] + (["TE", "ED"] if case.turb_model == 1 else [])
        for nm in fields:
            err = _rel_l2(srv.result_field(ids[n], nm, case.ncel), o.get(nm))
            assert err < 1e-8, f"{n} {nm}: relative L2 {err:.3e}"
        o.close()
    srv.close()
