"""The bench workload itself: the k-epsilon channel of 200x20x20 hexes cut into 6 tets each,
interior nodes jittered by 0.15h (seed 2026) -- 480000 cells, 976800 faces.

At this size the oracle still runs single stages in seconds, so the parity bar of the small
cases holds here too: geometry, the CSR pattern and every assembly and correction stage are
bit-exact against the oracle on the same inputs (the state after two GPU iterations, copied
into the oracle).  The Krylov solves are checked through properties that do not depend on a
reference run: the left-preconditioned GMRES stopping test ||M^-1 (b - A x)|| <= rtol ||M^-1 b||
recomputed on the CPU from the returned solution (M^-1 the degree-2 Jacobi-Neumann polynomial,
rebuilt here from A), and the pressure CG's true residual.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi, meshgen
from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver

pytestmark = pytest.mark.gpu

GEOM = ["face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "face_xpac", "face_xnac", "cell_vol",
        "cell_x", "bnd_distance"]
STATE = ["U", "V", "W", "P", "R", "VisLam", "VisTur", "Apr", "deltaP", "RUFace", "BRo", "BU", "BV", "BW", "BPre",
         "TE", "ED", "BTE", "BED"]


@pytest.fixture(scope="module")
def bench_pair(tmp_path_factory):
    d = tmp_path_factory.mktemp("channel480k")
    param = meshgen.write_case(str(d), "channel", nx=200, ny=20, nz=20, jitter=0.15, seed=2026, steps=10)
    opt = capi.default_options(pc=capi.PC_POLY2)
    opt.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    g = NavierStokesSolver(Case(param), opt)
    o = po.OracleCase(param)
    return o, g


def _bits_equal(a, b):
    return np.array_equal(a.view(np.int64), b.view(np.int64))


def test_bench_case_size(bench_pair):
    o, g = bench_pair
    assert g.case.ncel == 480000 and o.ncel == 480000


def test_geometry_and_pattern_bit_exact(bench_pair):
    o, g = bench_pair
    for nm in GEOM:
        a, b = g.get(nm), o.get(nm)
        assert _bits_equal(a, b), f"{nm}: max |diff| {np.max(np.abs(a - b))}"
    assert np.array_equal(g.get_int("A_rowptr"), o.geti("A_rowptr"))
    assert np.array_equal(g.get_int("A_col"), o.geti("A_col"))


def test_assembly_and_correction_stages_bit_exact(bench_pair):
    o, g = bench_pair
    g.iterate(2)  # a developed state, copied into the oracle
    for nm in STATE:
        o.set(nm, g.get(nm))
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
    dp = np.random.default_rng(3).standard_normal(o.ncel) * 1e-3
    o.set("deltaP", dp)
    g.set("deltaP", dp)
    for stage, outputs in [("bc_deltap", ["BPre"]), ("grad_deltap", ["dPdX"]),
                           ("correct_cells", ["P", "U", "V", "W"]), ("bc_velocity", ["BU", "BV", "BW", "BRo"]),
                           ("correct_ruface", ["RUFace"])]:
        o.stage(stage)
        g.stage(stage)
        for nm in outputs:
            a, b = g.get(nm), o.get(nm)
            assert _bits_equal(a, b), f"{stage}/{nm}: max |diff| {np.max(np.abs(a - b))}"


def test_keps_stages_bit_exact_at_full_size(bench_pair):
    from test_gpu_parity import _keps_stages_bit_exact
    o, g = bench_pair
    g.iterate(1)
    for nm in STATE + ["dUdX", "dVdX", "dWdX"]:
        o.set(nm, g.get(nm))
    _keps_stages_bit_exact(o, g)


def _csr(g, name):
    n = g.case.ncel
    return sp.csr_matrix((g.get(name), g.get_int("A_col"), g.get_int("A_rowptr")), shape=(n, n))


def test_gmres_stopping_test_holds_at_full_size(bench_pair):
    """u, v, w solved by GMRES(30) with the degree-2 polynomial: the returned solutions satisfy
    the left-preconditioned stopping test, recomputed here from A and b."""
    o, g = bench_pair
    g.stage("build_velocity")
    A = _csr(g, "Au_val")
    dinv = 1.0 / A.diagonal()

    def minv(y):  # sum_{i<=2} (I - D^-1 A)^i D^-1 y
        z = dinv * y
        s = z.copy()
        for _ in range(2):
            s = z + s - dinv * (A @ s)
        return s

    rtol = 1e-8
    xs = [g.get(nm).copy() for nm in ("U", "V", "W")]
    bs = [g.get(nm) for nm in ("bu", "bv", "bw")]
    g.solveVelocity_GMRES(rtol, 1000, *xs)
    for x, b in zip(xs, bs):
        r = minv(b - A @ x)
        ref = np.linalg.norm(minv(b))
        assert np.linalg.norm(r) <= 1.01 * rtol * ref, (np.linalg.norm(r), rtol * ref)


def test_pressure_cg_true_residual_at_full_size(bench_pair):
    o, g = bench_pair
    g.stage("build_velocity")
    g.stage("ruface2")
    g.stage("build_pressure")
    A = _csr(g, "Ap_val")
    b = g.get("bp")
    x = np.zeros(g.case.ncel)
    g.solvePressureCorrection(1e-12, 1000, x)
    rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert rel < 1e-8, rel
