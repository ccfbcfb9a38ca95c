"""Transient runs, the energy equation and the perfect-gas (DensityModel 1) branches against the
oracle (NS/navier.cpp:52-111, navier_scalar.cpp:204-326, navier_pressure.cpp with DensityModel 1).

Stages on identical inputs are bit-exact, as on the steady path: momentum rows with their
unsteady terms, the compressible pressure-correction rows, the density and flux corrections,
and the assembled energy system.  Whole time steps agree like two runs of the same algorithm:
the same number of outer iterations, residual histories to relative 1e-6, Krylov iteration
counts within one, fields to relative L2 1e-8.
"""
import os

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi, meshgen
from sysu_cfd_parallel_gb300.solver import Batch, Case, NavierStokesSolver

pytestmark = pytest.mark.gpu

CASES = {
    "cav_euler": ("cavity", dict(n=6, time=(0.05, 1.0, 20, "Euler"))),
    "cav_dual": ("cavity", dict(n=6, jitter=0.1, seed=4, time=(0.05, 1.0, 20, "Dual"))),
    "cav_energy": ("cavity", dict(n=7, energy=True, wall_t=300, lid_t=320)),
    "cav_gas": ("cavity", dict(n=6, density=1, wall_t=300, lid_t=320)),
    "cav_gas_tr": ("cavity", dict(n=6, jitter=0.1, seed=5, density=1, wall_t=300, lid_t=330,
                                  time=(0.05, 1.0, 20, "Euler"))),
    "ch_tr_energy": ("channel", dict(nx=10, ny=2, nz=2, time=(0.1, 1.0, 10, "Dual"), energy=True, wall_t=290,
                                     t_in=300)),
}


@pytest.fixture(scope="module")
def tcase(tmp_path_factory):
    root = tmp_path_factory.mktemp("transient")
    made = {}

    def get(name):
        if name not in made:
            kind, kw = CASES[name]
            made[name] = meshgen.write_case(str(root / name), kind, **kw)
        return made[name]

    return get


def _pair(param):
    o = po.OracleCase(param)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, po.PC_JACOBI, 30)
    g = NavierStokesSolver(Case(param), capi.default_options(pc=capi.PC_JACOBI))
    return o, g


def _bits_equal(a, b):
    return np.array_equal(a.view(np.int64), b.view(np.int64))


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


STATE = ["U", "V", "W", "P", "R", "T", "VisLam", "VisTur", "Apr", "deltaP", "RUFace", "BRo", "BU", "BV", "BW",
         "BPre", "BTem", "dUdX", "dVdX", "dWdX", "dPdX"]


def _copy_state(o, g, names):
    for nm in names:
        g.set(nm, o.get(nm))


def test_case_physics_read_from_param(tcase):
    c = Case(tcase("cav_dual"))
    assert not c.steady and c.time_scheme == 2 and c.max_outer == 20 and c.dt == 0.05
    assert c.max_step == int(1.0 / 0.05)
    g = Case(tcase("cav_gas"))
    assert g.density_model == 1 and g.solve_energy and g.steady
    # perfect-gas initial density, as the oracle computes it
    o = po.OracleCase(tcase("cav_gas"))
    assert _bits_equal(g.get_field("R"), o.get("R"))


@pytest.mark.parametrize("name", ["cav_euler", "cav_dual", "cav_gas_tr"])
def test_unsteady_momentum_rows_bit_exact(tcase, name):
    o, g = _pair(tcase(name))
    o.time_step()  # a non-trivial state with a previous time level
    _copy_state(o, g, STATE)
    for nm in ("Rnp", "Unp", "Vnp", "Wnp", "Tnp"):
        g.set(nm, o.get(nm))
    o.stage("build_velocity")
    g.stage("build_velocity")
    for nm in ("Au_val", "bu", "bv", "bw", "Apr"):
        a, b = g.get(nm), o.get(nm)
        assert _bits_equal(a, b), f"{nm}: max |diff| {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("name", ["cav_gas", "cav_gas_tr"])
def test_gas_pressure_and_corrections_bit_exact(tcase, name):
    o, g = _pair(tcase(name))
    if o.physics()["steady"]:
        o.iterate(2)
    else:
        o.time_step()
    _copy_state(o, g, STATE)
    for stage, outputs in [("ruface2", ["RUFace"]), ("build_pressure", ["Ap_val", "bp"])]:
        o.stage(stage)
        g.stage(stage)
        for nm in outputs:
            a, b = g.get(nm), o.get(nm)
            assert _bits_equal(a, b), f"{stage}/{nm}: max |diff| {np.max(np.abs(a - b))}"
    dp = np.random.default_rng(1).standard_normal(o.ncel) * 1e-2
    o.set("deltaP", dp)
    g.set("deltaP", dp)
    for stage, outputs in [("bc_deltap", ["BPre"]), ("grad_deltap", ["dPdX"]),
                           ("correct_cells", ["P", "R", "U", "V", "W"]), ("bc_velocity", ["BU", "BV", "BW", "BRo"]),
                           ("correct_ruface", ["RUFace"])]:
        o.stage(stage)
        g.stage(stage)
        for nm in outputs:
            a, b = g.get(nm), o.get(nm)
            assert _bits_equal(a, b), f"{stage}/{nm}: max |diff| {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("name", ["cav_energy", "cav_gas", "cav_gas_tr", "ch_tr_energy"])
def test_energy_system_bit_exact(tcase, name):
    o, g = _pair(tcase(name))
    if o.physics()["steady"]:
        o.iterate(2)
    else:
        o.time_step()
    names = STATE + (["TE", "ED", "BTE", "BED"] if o.turb == 1 else [])
    _copy_state(o, g, names)
    if not o.physics()["steady"]:
        g.set("Tnp", o.get("Tnp"))
    o.stage("build_energy")
    g.stage("build_energy")
    for nm in ("kcond", "ESource", "ApE", "BTem", "dPhidX", "As_val", "bs"):
        a, b = g.get(nm), o.get(nm)
        assert _bits_equal(a, b), f"{nm}: max |diff| {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("name,steps", [("cav_euler", 3), ("cav_dual", 3), ("cav_gas_tr", 2), ("ch_tr_energy", 2)])
def test_time_steps_match_oracle(tcase, name, steps):
    o, g = _pair(tcase(name))
    for _ in range(steps):
        ro = o.time_step()
        rg = g.time_step()
        assert rg["n"] == ro["n"], (rg["n"], ro["n"])
        np.testing.assert_allclose(rg["resmax"], ro["resmax"], rtol=1e-6)
        assert np.all(np.abs(rg["ksp_its"] - ro["ksp_its"]) <= 1), (rg["ksp_its"], ro["ksp_its"])
    fields = ["U", "V", "W", "P", "T", "R"] + (["TE", "ED"] if o.turb == 1 else [])
    for nm in fields:
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"
    assert abs(g.cur_time - o.physics()["cur_time"]) < 1e-12


@pytest.mark.parametrize("name,steps", [("cav_energy", 6), ("cav_gas", 4)])
def test_steady_energy_and_gas_iterations_match_oracle(tcase, name, steps):
    o, g = _pair(tcase(name))
    ro = o.iterate(steps)
    rg = g.iterate(steps)
    assert np.all(np.abs(rg["ksp_its"] - ro["ksp_its"]) <= 1), (rg["ksp_its"], ro["ksp_its"])
    np.testing.assert_allclose(rg["resmax"], ro["resmax"], rtol=1e-6)
    for nm in ("U", "V", "W", "P", "T", "R"):
        err = _rel_l2(g.get(nm), o.get(nm))
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


def test_transient_nssolve_and_graph_replay(tcase, tmp_path):
    p = tcase("cav_euler")
    a = NavierStokesSolver(Case(p), capi.default_options(pc=capi.PC_JACOBI))
    b = NavierStokesSolver(Case(p), capi.default_options(pc=capi.PC_JACOBI))
    b.set_graph(True)
    seen = []
    a.NSSolve(max_step=3, callback=lambda s, rm, res: seen.append(s), output_dir=str(tmp_path))
    for _ in range(3):
        b.time_step()
    assert seen == [1, 2, 3] and abs(a.cur_time - 0.15) < 1e-12
    for nm in ("U", "V", "W", "P"):
        assert _bits_equal(a.get(nm), b.get(nm)), nm
    assert os.path.exists(tmp_path / "tec" / "res0000.dat")


def test_batches_refuse_transient_and_gas(tcase, cases):
    with pytest.raises(capi.CycasError):
        Batch([Case(tcase("cav_euler")), Case(cases("cavity4"))])
    with pytest.raises(capi.CycasError):
        Batch([Case(tcase("cav_gas"))])
    s = NavierStokesSolver(Case(cases("cavity4")), capi.default_options(pc=capi.PC_JACOBI))
    with pytest.raises(capi.CycasError):
        s.time_step()
