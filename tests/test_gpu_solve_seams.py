"""DataPartition::solve* mirrors (cycas_solve_velocity / _pressure / _scalar) against the oracle's
Krylov solver on the same assembled systems (MPIStructure.cpp:234-531).

The context assembles the rows (bit-exact with the oracle, see test_gpu_parity), the caller's host
arrays are solved in place, and the oracle solves the same CSR system from the same initial guess:
solutions agree to relative L2 1e-8 and iteration counts within one, as for any two runs of the
same Krylov method whose inner products sum in different orders.  The context's own fields are
left untouched.
"""
import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import Case, ConvergeError, NavierStokesSolver

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


def _setup(param):
    o = po.OracleCase(param)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, po.PC_JACOBI, 30)
    o.iterate(2)
    g = NavierStokesSolver(Case(param), capi.default_options(pc=capi.PC_JACOBI))
    names = ["U", "V", "W", "P", "R", "VisLam", "VisTur", "Apr", "RUFace", "BRo", "BU", "BV", "BW", "BPre"]
    if o.turb == 1:
        names += ["TE", "ED", "BTE", "BED"]
    for nm in names:
        g.set(nm, o.get(nm))
    return o, g


def test_velocity_pressure_scalar_seams(cases):
    o, g = _setup(cases("channel_small"))
    rp, col = g.get_int("A_rowptr"), g.get_int("A_col")
    g.stage("build_velocity")
    val = g.get("Au_val")
    x0 = [g.get(nm) for nm in ("U", "V", "W")]
    xs = [x.copy() for x in x0]
    st = g.solveVelocity_GMRES(1e-8, 1000, *xs)
    for q, b in enumerate(("bu", "bv", "bw")):
        xr, its, reason, _ = po.csr_solve(rp, col, val, g.get(b), x0=x0[q], pc=po.PC_JACOBI, rtol=1e-8, maxit=1000,
                                          guess_zero=False)
        assert reason > 0 and st.reason[q] > 0
        assert abs(st.its[q] - its) <= 1, (st.its[q], its)
        assert _rel_l2(xs[q], xr) < 1e-8
    for q, nm in enumerate(("U", "V", "W")):  # the context's own fields are untouched
        assert np.array_equal(g.get(nm), x0[q])

    g.stage("ruface2")
    g.stage("build_pressure")
    val, bp = g.get("Ap_val"), g.get("bp")
    for sym, kt in ((True, po.KSP_CG), (False, po.KSP_GMRES)):
        xp = np.full(g.case.ncel, 3.0)  # the guess is ignored: the reference solves from zero
        st = g.solvePressureCorrection(1e-6, 1000, xp, sym)
        xr, its, reason, _ = po.csr_solve(rp, col, val, bp, pc=po.PC_JACOBI, rtol=1e-6, maxit=1000, ksp_type=kt)
        assert abs(st.its[0] - its) <= 1, (sym, st.its[0], its)
        assert _rel_l2(xp, xr) < 1e-8

    g.stage("keps")  # leaves the epsilon rows in As / bs
    val, bs = g.get("As_val"), g.get("bs")
    ed = np.random.default_rng(2).random(g.case.ncel) * 1e-3
    xs = ed.copy()
    st = g.solveScarlar_GMRES(1e-8, 500, xs)
    xr, its, reason, _ = po.csr_solve(rp, col, val, bs, x0=ed, pc=po.PC_JACOBI, rtol=1e-8, maxit=500,
                                      guess_zero=False)
    assert abs(st.its[0] - its) <= 1
    assert _rel_l2(xs, xr) < 1e-8


def test_seam_reports_non_convergence(cases):
    o, g = _setup(cases("cavity8"))
    g.stage("build_velocity")
    xs = [g.get(nm) for nm in ("U", "V", "W")]
    with pytest.raises(ConvergeError):
        g.solveVelocity_GMRES(1e-14, 1, *xs)
    with pytest.raises(capi.CycasError):
        g.solveScarlar_GMRES(-1.0, 10, xs[0])


def test_set_and_get_fields_in_one_call(cases):
    g = NavierStokesSolver(Case(cases("channel_tiny")), capi.default_options(pc=capi.PC_JACOBI))
    n = g.case.ncel
    rng = np.random.default_rng(5)
    vals = {nm: rng.standard_normal(n) for nm in ("U", "V", "W", "P", "TE")}
    g.set_fields(vals)
    for nm, v in vals.items():
        assert np.array_equal(g.get(nm), v), nm
    out = {nm: np.empty(n) for nm in vals}
    g.get_fields(out)
    for nm in vals:
        assert np.array_equal(out[nm], vals[nm]), nm
    # a bad size anywhere rejects the whole call before anything is copied
    bad = {"U": np.zeros(n), "V": np.zeros(n - 1)}
    with pytest.raises(capi.CycasError):
        g.set_fields(bad)
    assert np.array_equal(g.get("U"), vals["U"])


@pytest.mark.parametrize("name", ["channel_small", "cavity8"])
def test_iteration_with_host_io_matches_separate_calls(cases, name):
    """cycas_simple_iteration_io (uploads and downloads overlapping the iteration) gives the
    results of cycas_set_fields + cycas_simple_iteration + cycas_get_fields, bit for bit, with
    the same host arrays as input and output."""
    p = cases(name)
    a = NavierStokesSolver(Case(p), capi.default_options(pc=capi.PC_JACOBI))
    b = NavierStokesSolver(Case(p), capi.default_options(pc=capi.PC_JACOBI))
    turb = a.case.turb_model == 1
    names_in = ["U", "V", "W", "P", "R", "VisLam", "VisTur", "RUFace", "BRo", "BU", "BV", "BW"]
    names_out = ["U", "V", "W", "P", "VisTur", "RUFace"]
    if turb:
        names_in += ["TE", "ED", "BTE", "BED"]
        names_out += ["TE", "ED"]
    ha = {nm: a.get(nm).copy() for nm in set(names_in) | set(names_out)}
    hb = {nm: v.copy() for nm, v in ha.items()}
    rng = np.random.default_rng(11)
    for nm in ("U", "V", "W"):  # a host-side change the device must pick up every iteration
        ha[nm] += 1e-3 * rng.standard_normal(ha[nm].size)
        hb[nm][:] = ha[nm]
    for _ in range(3):
        ra = a.simple_iteration_io({nm: ha[nm] for nm in names_in}, {nm: ha[nm] for nm in names_out})
        b.set_fields({nm: hb[nm] for nm in names_in})
        rb = b.simple_iteration()
        b.get_fields({nm: hb[nm] for nm in names_out})
        assert ra == rb
        assert np.array_equal(a.Residual, b.Residual)
        for nm in names_out:
            assert np.array_equal(ha[nm].view(np.int64), hb[nm].view(np.int64)), nm
        ha["U"] *= 1.0001  # perturb between iterations, as a coupled caller would
        hb["U"][:] = ha["U"]
