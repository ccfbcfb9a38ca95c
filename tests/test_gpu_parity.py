"""GPU path (libcycasgpu through the C ABI) against the CPU oracle.

Bit-exact: geometry, gradients, momentum / pressure / scalar assembly, Rhie-Chow and
corrections are per-cell gathers rounded exactly as the reference's source orders them,
so on identical inputs they must agree to the last bit with the oracle (built with
-ffp-contract=off).  Krylov solves reduce in a different order, so whole iterations are
compared with tolerances: fields to relative L2 1e-8 after the solves converge to
rtol, residual histories to relative 1e-6, iteration counts within one.
"""
import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver

pytestmark = pytest.mark.gpu

GEOM = ["face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "face_xpac", "face_xnac", "cell_vol",
        "cell_x", "bnd_distance"]
STATE = ["U", "V", "W", "P", "R", "VisLam", "VisTur", "Apr", "deltaP", "RUFace", "BRo", "BU", "BV", "BW", "BPre"]
STATE_KE = ["TE", "ED", "BTE", "BED"]


def _pair(param, pc=po.PC_JACOBI, restart=30):
    o = po.OracleCase(param)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, pc, restart)
    g = NavierStokesSolver(Case(param), capi.default_options(pc=capi.PC_JACOBI if pc == po.PC_JACOBI else pc,
                                                             restart=restart))
    return o, g


def _copy_state(o, g, turb):
    for nm in STATE + (STATE_KE if turb else []):
        g.set(nm, o.get(nm))


def _bits_equal(a, b):
    return np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("name", ["cavity4", "cavity8j", "channel_tiny", "channel_small"])
def test_geometry_bit_exact(cases, name):
    o, g = _pair(cases(name))
    for nm in GEOM:
        a, b = g.get(nm), o.get(nm)
        assert _bits_equal(a, b), f"{nm}: max |diff| {np.max(np.abs(a - b))}"
    assert np.array_equal(g.get_int("A_rowptr"), o.geti("A_rowptr"))
    assert np.array_equal(g.get_int("A_col"), o.geti("A_col"))


KEPS_TE = ["Prod", "TESource", "ApTE", "VisTE", "VisED", "BTE", "BED", "ED", "dPhidX", "As_val", "bs"]
KEPS_ED = ["TE", "EDSource", "ApED", "dPhidX", "As_val", "bs"]


def _keps_stages_bit_exact(o, g):
    """k rows, then epsilon rows on a k both sides share (the GPU's k after its own solve)."""
    o.stage("build_te")
    g.stage("build_te")
    for nm in KEPS_TE:
        a, b = g.get(nm), o.get(nm)
        assert _bits_equal(a, b), f"build_te/{nm}: max |diff| {np.max(np.abs(a - b))}"
    te = np.abs(np.random.default_rng(7).standard_normal(o.ncel)) * np.mean(np.abs(o.get("TE")))
    te[::97] = 1e-12  # below the clip
    o.set("TE", te)
    g.set("TE", te)
    o.stage("build_ed")
    g.stage("build_ed")
    for nm in KEPS_ED:
        a, b = g.get(nm), o.get(nm)
        assert _bits_equal(a, b), f"build_ed/{nm}: max |diff| {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("name", ["channel_tiny", "channel_small"])
def test_keps_stages_bit_exact(cases, name):
    o, g = _pair(cases(name))
    o.iterate(3)
    _copy_state(o, g, True)
    for nm in ("dUdX", "dVdX", "dWdX"):
        g.set(nm, o.get(nm))
    _keps_stages_bit_exact(o, g)


@pytest.mark.parametrize("name", ["cavity8", "channel_small"])
def test_assembly_stages_bit_exact(cases, name):
    o, g = _pair(cases(name))
    o.iterate(3)  # a non-trivial state
    turb = o.turb == 1
    _copy_state(o, g, turb)
    for stage, outputs in [
        ("build_velocity", ["BRo", "BU", "BV", "BW", "BPre", "dUdX", "dVdX", "dWdX", "dPdX", "Au_val", "bu", "bv",
                            "bw", "Apr", "bnd_shear"]),
        ("ruface2", ["RUFace"]),
        ("build_pressure", ["Ap_val", "bp"]),
    ]:
        o.stage(stage)
        g.stage(stage)
        for nm in outputs:
            a, b = g.get(nm), o.get(nm)
            assert _bits_equal(a, b), f"{stage}/{nm}: max |diff| {np.max(np.abs(a - b))}"
    # correction stages on a shared pressure-correction field
    dp = np.random.default_rng(0).standard_normal(o.ncel) * 1e-3
    o.set("deltaP", dp)
    g.set("deltaP", dp)
    for stage, outputs in [("bc_deltap", ["BPre"]), ("grad_deltap", ["dPdX"]),
                           ("correct_cells", ["P", "U", "V", "W"]), ("bc_velocity", ["BU", "BV", "BW", "BRo"]),
                           ("correct_ruface", ["RUFace"])]:
        if stage == "bc_deltap":
            o.stage("bc_deltap")
        else:
            o.stage(stage)
        g.stage(stage)
        for nm in outputs:
            a, b = g.get(nm), o.get(nm)
            assert _bits_equal(a, b), f"{stage}/{nm}: max |diff| {np.max(np.abs(a - b))}"


def _rel_l2(a, b):
    d = np.linalg.norm(a - b)
    s = np.linalg.norm(b)
    return d / s if s > 0 else d


@pytest.mark.parametrize("name,steps", [("cavity8", 15), ("cavity8j", 10), ("channel_tiny", 6)])
def test_iterations_match_oracle(cases, name, steps):
    o, g = _pair(cases(name))
    ro = o.iterate(steps)
    rg = g.iterate(steps)
    # Krylov iteration counts: same algorithm, reductions in a different order
    assert np.all(np.abs(rg["ksp_its"] - ro["ksp_its"]) <= 1), (rg["ksp_its"], ro["ksp_its"])
    np.testing.assert_allclose(rg["resmax"], ro["resmax"], rtol=1e-6)
    fields = ["U", "V", "W", "P"] + (["TE", "ED"] if o.turb == 1 else [])
    for nm in fields:
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


def test_full_grid_iterations_match_oracle(cases):
    """46k cells: every persistent kernel runs on all SMs (the grid size of the small cases
    is a handful of CTAs)."""
    o, g = _pair(cases("cavity36"))
    ro = o.iterate(2)
    rg = g.iterate(2)
    assert np.all(np.abs(rg["ksp_its"] - ro["ksp_its"]) <= 1), (rg["ksp_its"], ro["ksp_its"])
    for nm in ("U", "V", "W", "P"):
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


def test_csr_gmres_matches_oracle():
    from sysu_cfd_parallel_gb300.solver import csr_solve
    rng = np.random.default_rng(1)
    n = 3000
    # nonsymmetric, diagonally dominant 7-band system
    offs = [-40, -7, -1, 0, 1, 7, 40]
    rows, cols, vals = [], [], []
    for i in range(n):
        for o_ in offs:
            j = i + o_
            if 0 <= j < n:
                rows.append(i); cols.append(j)
                vals.append(8.0 + rng.random() if o_ == 0 else -rng.random())
    rows = np.array(rows); cols = np.array(cols); vals = np.array(vals)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, dtype=np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    b = rng.standard_normal(n)
    xg, itg, rg_, _ = csr_solve(rowptr, cols, vals, b, rtol=1e-10, restart=20)
    xo, ito, ro_, _ = po.csr_solve(rowptr, cols, vals, b, rtol=1e-10, restart=20)
    assert rg_ > 0 and ro_ > 0
    assert abs(itg - ito) <= 1
    assert _rel_l2(xg, xo) < 1e-9


def _opts(pressure_pc, rtol_p=0.0, rtol_v=0.0):
    o = capi.default_options(pc=capi.PC_JACOBI)
    o.ksp[capi.SYS_PRESSURE].pc = pressure_pc
    o.ksp[capi.SYS_PRESSURE].rtol = rtol_p
    for s in (capi.SYS_VELOCITY, capi.SYS_SCALAR):
        o.ksp[s].rtol = rtol_v
    return o


@pytest.mark.parametrize("name,steps", [("cavity8", 6), ("channel_small", 4)])
def test_amg_pressure_matches_reference_ilu(cases, name, steps):
    """Pressure CG with the AMG V-cycle vs the reference's ILU(0)-CG, both solved tightly:
    the preconditioner changes the Krylov path, not the solution."""
    p = cases(name)
    o = po.OracleCase(p)
    o.set_ksp(po.VELOCITY, po.PC_JACOBI, rtol=1e-12)
    o.set_ksp(po.SCALAR, po.PC_JACOBI, rtol=1e-12)
    o.set_ksp(po.PRESSURE, po.PC_ILU0, rtol=1e-12, ksp_type=po.KSP_CG)
    g = NavierStokesSolver(Case(p), _opts(capi.PC_AMG, rtol_p=1e-12, rtol_v=1e-12))
    o.iterate(steps)
    rg = g.iterate(steps)
    assert np.all(rg["ksp_reason"][:, :4] > 0)
    fields = ["U", "V", "W", "P"] + (["TE", "ED"] if o.turb == 1 else [])
    for nm in fields:
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


@pytest.mark.parametrize("name,steps,gamma,omega", [("cavity8", 4, 2, 0.0), ("channel_small", 3, 3, 0.0),
                                                   ("cavity8j", 3, 1, 2.0 / 3.0)])
def test_amg_cycle_options_match_reference_ilu(cases, name, steps, gamma, omega):
    """The cycle's options (several cycles at the first shared-memory level -- which these
    small cases only take when asked --, another smoother weight) change the Krylov path, not
    the solution: tight solves agree with the reference's ILU(0)-CG."""
    p = cases(name)
    o = po.OracleCase(p)
    o.set_ksp(po.VELOCITY, po.PC_JACOBI, rtol=1e-12)
    o.set_ksp(po.SCALAR, po.PC_JACOBI, rtol=1e-12)
    o.set_ksp(po.PRESSURE, po.PC_ILU0, rtol=1e-12, ksp_type=po.KSP_CG)
    opt = _opts(capi.PC_AMG, rtol_p=1e-12, rtol_v=1e-12)
    opt.amg_gamma = gamma
    opt.amg_omega = omega
    g = NavierStokesSolver(Case(p), opt)
    o.iterate(steps)
    rg = g.iterate(steps)
    assert np.all(rg["ksp_reason"][:, :4] > 0)
    fields = ["U", "V", "W", "P"] + (["TE", "ED"] if o.turb == 1 else [])
    for nm in fields:
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


def test_amg_w_cycle_cuts_iterations(cases):
    p = cases("channel_small")
    its = {}
    for gamma in (1, 2):
        opt = _opts(capi.PC_AMG)
        opt.amg_gamma = gamma
        r = NavierStokesSolver(Case(p), opt).iterate(3)
        assert np.all(r["ksp_reason"][:, 3] > 0)
        its[gamma] = int(r["ksp_its"][:, 3].sum())
    assert its[2] < its[1], its


def test_amg_options_out_of_range_rejected(cases):
    p = cases("cavity4")
    for field, value in (("amg_alpha", 2.5), ("amg_omega", 1.2), ("amg_gamma", 5)):
        opt = _opts(capi.PC_AMG)
        setattr(opt, field, value)
        with pytest.raises(capi.CycasError):
            NavierStokesSolver(Case(p), opt)


def test_amg_cuts_pressure_iterations(cases):
    p = cases("channel_small")
    g1 = NavierStokesSolver(Case(p), _opts(capi.PC_JACOBI))
    g2 = NavierStokesSolver(Case(p), _opts(capi.PC_AMG))
    r1 = g1.iterate(3)
    r2 = g2.iterate(3)
    assert np.all(r2["ksp_reason"][:, 3] > 0)
    assert r2["ksp_its"][:, 3].max() * 3 < r1["ksp_its"][:, 3].min()


@pytest.mark.parametrize("name,steps,poly", [("cavity8j", 8, 1), ("channel_small", 5, 1), ("channel_small", 4, 2),
                                             ("cavity8j", 6, 3), ("channel_small", 4, 3), ("channel_small", 4, 5),
                                             ("cavity8j", 5, 5)])
def test_polynomial_preconditioner_matches_oracle(cases, name, steps, poly):
    """GMRES with the Jacobi-Neumann polynomial preconditioner (momentum and scalars; CG with
    Jacobi for the pressure correction), GPU against the oracle's restatement of it."""
    p = cases(name)
    opc = {1: po.PC_POLY1, 2: po.PC_POLY2, 3: po.PC_POLY3, 5: po.PC_POLY5}[poly]
    gpc = {1: capi.PC_POLY1, 2: capi.PC_POLY2, 3: capi.PC_POLY3, 5: capi.PC_POLY5}[poly]
    o = po.OracleCase(p)
    o.set_ksp(po.VELOCITY, opc, 30)
    o.set_ksp(po.PRESSURE, po.PC_JACOBI, 30)
    o.set_ksp(po.SCALAR, opc, 30)
    opts = capi.default_options(pc=capi.PC_JACOBI)
    opts.ksp[capi.SYS_VELOCITY].pc = gpc
    opts.ksp[capi.SYS_SCALAR].pc = gpc
    g = NavierStokesSolver(Case(p), opts)
    ro = o.iterate(steps)
    rg = g.iterate(steps)
    assert np.all(np.abs(rg["ksp_its"] - ro["ksp_its"]) <= 1), (rg["ksp_its"], ro["ksp_its"])
    np.testing.assert_allclose(rg["resmax"], ro["resmax"], rtol=1e-6)
    for nm in ["U", "V", "W", "P"] + (["TE", "ED"] if o.turb == 1 else []):
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


def test_polynomial_preconditioner_nonzero_guess_csr(cases):
    """The standalone solve with a nonzero initial guess: |M^-1 b| is the reference norm."""
    from sysu_cfd_parallel_gb300.solver import csr_solve
    o, g = _pair(cases("channel_small"))
    o.iterate(2)
    _copy_state(o, g, True)
    g.stage("build_velocity")
    rp, col, val, b = g.get_int("A_rowptr"), g.get_int("A_col"), g.get("Au_val"), g.get("bu")
    x0 = g.get("U")
    xr, its_r, reason_r, _ = po.csr_solve(rp, col, val, b, x0=x0, pc=po.PC_POLY2, rtol=1e-8, maxit=1000,
                                          guess_zero=False)
    xg, its_g, reason_g, _ = csr_solve(rp, col, val, b, x0=x0, pc=capi.PC_POLY2, rtol=1e-8, guess_zero=False)
    assert reason_r > 0 and reason_g > 0 and abs(its_g - its_r) <= 1, (its_g, its_r)
    assert _rel_l2(xg, xr) < 1e-8
