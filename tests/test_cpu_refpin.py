"""The oracle against the reference's own code (CPU).

tests/golden/*/ref_{ilu,jacobi}.npz were written by the reference's unmodified solver sources,
built single-rank by oracle/refpin (tests/golden/make_ref_golden.py).  Both sides run their
Krylov solves through the same restatement of PETSc's algorithms (oracle/oracle_krylov.cpp), so
everything else -- mesh ingest and sort, face discovery, geometry, boundary conditions,
gradients, the momentum / pressure / k-epsilon / energy assembly, corrections, residuals, the
outer loop -- is the reference's own arithmetic on one side and the restatement on the other,
and must agree bit for bit.  The oracle takes TE^1.5 of the wall function through the C
library's pow here, as the reference does (its default is the once-rounded value the GPU
computes; test_pow15_differs_from_libm_by_one_ulp_at_most covers the difference).

Unused slots are not compared: the reference leaves Cell.face/cell beyond nface at INT_MAX and
Face.Xpac/Xnac of boundary faces at DBL_MAX (its constructors' fill values, never read); the
oracle stores -1 and 0 there.
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, GOLDEN)

import pyoracle as po  # noqa: E402

CASES = ["cavity5j", "channel_tiny", "cavity5g_dual", "channel_tiny_tr"]
INT_ARRAYS = ["face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "bnd_face", "bnd_rid",
              "cell_vertices", "bnd_vertices"]
GEOMETRY = ["face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "cell_vol", "cell_x", "bnd_distance"]
PCS = {"ilu": po.PC_ILU0, "jacobi": po.PC_JACOBI}


def _oracle(param, pc, ksp_gmres_all=False, rtol=None):
    o = po.OracleCase(param)
    o.set_libm_pow(True)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, PCS[pc], 30, -1.0 if rtol is None else rtol,
                  ksp_type=po.KSP_GMRES if ksp_gmres_all else None)
    return o


def _run(o, steps, transient):
    """Residual history [outer iterations, 10] and Krylov iterations of every solve."""
    if transient:
        rs = [o.time_step(cap=256) for _ in range(steps)]
        res = np.concatenate([r["residual"] for r in rs])
        its = np.concatenate([r["ksp_its"] for r in rs])
    else:
        r = o.iterate(steps)
        res, its = r["residual"], r["ksp_its"]
    return res, its[its >= 0]


@pytest.mark.parametrize("pc", ["ilu", "jacobi"])
@pytest.mark.parametrize("name", CASES)
def test_oracle_bit_exact_with_reference_build(name, pc):
    g = dict(np.load(os.path.join(GOLDEN, name, "ref_%s.npz" % pc)))
    param = os.path.join(GOLDEN, name, "param.in")
    o = _oracle(param, pc)
    for nm in INT_ARRAYS:
        assert np.array_equal(o.geti(nm), g[nm]), nm
    nface = g["cell_nface"]
    used = np.arange(6)[None, :] < nface[:, None]
    for nm in ("cell_face", "cell_cell"):
        a = o.geti(nm).reshape(-1, 6)
        assert np.array_equal(a[used], g[nm].reshape(-1, 6)[used]), nm
    for nm in GEOMETRY:
        assert np.array_equal(o.get(nm).view(np.int64), g[nm].view(np.int64)), nm
    interior = g["face_cell2"] >= 0
    for nm in ("face_xpac", "face_xnac"):
        a = o.get(nm).reshape(-1, 3)[interior]
        assert np.array_equal(a.view(np.int64), g[nm].reshape(-1, 3)[interior].view(np.int64)), nm
    transient = not o.physics()["steady"]
    res, its = _run(o, int(g["steps"]), transient)
    assert res.shape == g["residual"].shape
    assert np.array_equal(res.view(np.int64), g["residual"].view(np.int64)), np.abs(res - g["residual"]).max()
    assert np.array_equal(its, g["ksp"][:, 1].astype(np.int32))
    fields = ["U", "V", "W", "P", "R", "T", "VisTur", "RUFace", "deltaP", "Apr"]
    fields += ["TE", "ED"] if o.turb == 1 else []
    for nm in fields:
        assert np.array_equal(o.get(nm).view(np.int64), g[nm].view(np.int64)), nm
    o.close()


@pytest.mark.parametrize("pc", ["ilu", "jacobi"])
def test_cavity20_configured_run_bit_exact(pc, tmp_path):
    """The plain-method cavity for its configured 200 iterations, GMRES(30) rtol 1e-8 on every
    system (-ksp_type gmres -ksp_rtol 1e-8): residual history, every Krylov count and the final
    velocity and pressure equal the reference build's."""
    from make_ref_golden import write_cavity20
    g = dict(np.load(os.path.join(GOLDEN, "cavity20", "ref_%s.npz" % pc)))
    d = write_cavity20(str(tmp_path))
    o = _oracle(os.path.join(d, "param.in"), pc, ksp_gmres_all=True, rtol=1e-8)
    res, its = _run(o, 200, False)
    assert np.array_equal(res.view(np.int64), g["residual"].view(np.int64)), np.abs(res - g["residual"]).max()
    assert np.array_equal(its, g["ksp"][:, 1].astype(np.int32))
    for nm in ("U", "V", "W", "P"):
        assert np.array_equal(o.get(nm).view(np.int64), g[nm].view(np.int64)), nm
    o.close()


def test_cavity48_first_iterations_bit_exact(tmp_path):
    """The bench's cavity (48^3 hexahedra) for its first 5 SIMPLE iterations, ILU(0) and rtol
    1e-10 on every system: residual history, every Krylov count, and the L2 norm and sum of u, v,
    w, p equal the reference build's (tests/golden/cavity48/ref_ilu_tight.npz)."""
    from make_ref_golden import write_cavity48
    g = dict(np.load(os.path.join(GOLDEN, "cavity48", "ref_ilu_tight.npz")))
    d = write_cavity48(str(tmp_path))
    o = _oracle(os.path.join(d, "param.in"), "ilu", rtol=1e-10)
    res, its = _run(o, int(g["steps"]), False)
    assert np.array_equal(res.view(np.int64), g["residual"].view(np.int64)), np.abs(res - g["residual"]).max()
    assert np.array_equal(its, g["ksp"][:, 1].astype(np.int32))
    for nm in ("U", "V", "W", "P"):
        x = o.get(nm)
        assert np.linalg.norm(x) == g[nm + "_norm"] and np.sum(x) == g[nm + "_sum"], nm
    o.close()


def test_cavity48_reference_run_to_the_stop_test(tmp_path):
    """The reference build ran the bench's cavity to its own stop test (ResMax < 1e-6) at its own
    tolerances with ILU(0) (tests/golden/cavity48/ref_ilu_converged.npz): it stops at the first
    iteration below 1e-6, iteration 863 -- the iteration at which the GPU path with its own
    preconditioners stops too -- and its first iterations are the oracle's, bit for bit."""
    from sysu_cfd_parallel_gb300 import meshgen
    g = dict(np.load(os.path.join(GOLDEN, "cavity48", "ref_ilu_converged.npz")))
    rm = g["resmax"]
    assert len(rm) == 863 and rm[-1] < 1e-6 and np.all(rm[:-1] >= 1e-6)
    d = os.path.dirname(meshgen.write_case(str(tmp_path), "cavity", n=48, steps=3000, residual=1e-6))
    o = _oracle(os.path.join(d, "param.in"), "ilu")
    r = o.iterate(5)
    assert np.array_equal(np.asarray(r["resmax"]).view(np.int64), rm[:5].view(np.int64))
    o.close()


def test_batch_cavities_stop_where_the_reference_stops(tmp_path):
    """The batched workload's 256 cavities, each run by the reference build to its own stop test
    (tests/golden/batch_cavities/ref_stop.npz): the oracle stops the three smallest at the same
    SIMPLE iterations."""
    from make_ref_golden import batch_cavity_specs, write_batch_cavity
    g = dict(np.load(os.path.join(GOLDEN, "batch_cavities", "ref_stop.npz")))
    specs = batch_cavity_specs()
    assert len(g["case"]) == 256 and g["ref_stop"].sum() == 79640
    assert all(specs[k][:2] == (int(n), int(s)) for k, n, s in zip(g["case"], g["n"], g["seed"]))
    for i in range(3):
        k = int(g["case"][i])
        d = write_batch_cavity(str(tmp_path / str(k)), *specs[k])
        o = _oracle(os.path.join(d, "param.in"), "ilu")
        stop = None
        for it in range(1, 2 * int(g["ref_stop"][i])):
            if o.iterate(1)["resmax"][0] < 1e-6:
                stop = it
                break
        assert stop == int(g["ref_stop"][i]), (k, stop, int(g["ref_stop"][i]))
        o.close()


def test_channel_coarse_k_epsilon_bit_exact(tmp_path):
    """The configured k-epsilon channel's physics on a 7,500-tet jittered mesh for 10 SIMPLE
    iterations at the reference's tolerances with ILU(0): residual history, every Krylov count,
    and the L2 norm and sum of u, v, w, p, k, epsilon equal the reference build's
    (tests/golden/channel_coarse/ref_ilu.npz)."""
    from make_ref_golden import write_channel_coarse
    g = dict(np.load(os.path.join(GOLDEN, "channel_coarse", "ref_ilu.npz")))
    d = write_channel_coarse(str(tmp_path))
    o = _oracle(os.path.join(d, "param.in"), "ilu")
    res, its = _run(o, int(g["steps"]), False)
    assert np.array_equal(res.view(np.int64), g["residual"].view(np.int64)), np.abs(res - g["residual"]).max()
    assert np.array_equal(its, g["ksp"][:, 1].astype(np.int32))
    for nm in ("U", "V", "W", "P", "TE", "ED"):
        x = o.get(nm)
        assert np.linalg.norm(x) == g[nm + "_norm"] and np.sum(x) == g[nm + "_sum"], nm
    o.close()


def test_channel_coarse_transient_energy_bit_exact(tmp_path):
    """The same 7,500-tet channel run transient (Euler, dt 0.1) with the energy equation for 3
    time steps: the residual of every outer iteration, every Krylov count, and the L2 norm and
    sum of u, v, w, p, k, epsilon, T and rho equal the reference build's
    (tests/golden/channel_coarse_tr/ref_ilu.npz)."""
    from make_ref_golden import write_channel_coarse_tr
    g = dict(np.load(os.path.join(GOLDEN, "channel_coarse_tr", "ref_ilu.npz")))
    d = write_channel_coarse_tr(str(tmp_path))
    o = _oracle(os.path.join(d, "param.in"), "ilu")
    res, its = _run(o, int(g["steps"]), True)
    assert res.shape == g["residual"].shape
    assert np.array_equal(res.view(np.int64), g["residual"].view(np.int64)), np.abs(res - g["residual"]).max()
    assert np.array_equal(its, g["ksp"][:, 1].astype(np.int32))
    for nm in ("U", "V", "W", "P", "TE", "ED", "T", "R"):
        x = o.get(nm)
        assert np.linalg.norm(x) == g[nm + "_norm"] and np.sum(x) == g[nm + "_sum"], nm
    o.close()


def test_cavity16_perfect_gas_dual_bit_exact(tmp_path):
    """A perfect-gas cavity (16^3 hexahedra) with the reference's "Dual" scheme for 3 time steps:
    the residual of every outer iteration, every Krylov count, and the L2 norm and sum of u, v, w,
    p, T and rho equal the reference build's (tests/golden/cavity16g_dual/ref_ilu.npz)."""
    from make_ref_golden import write_cavity16g_dual
    g = dict(np.load(os.path.join(GOLDEN, "cavity16g_dual", "ref_ilu.npz")))
    d = write_cavity16g_dual(str(tmp_path))
    o = _oracle(os.path.join(d, "param.in"), "ilu")
    res, its = _run(o, int(g["steps"]), True)
    assert res.shape == g["residual"].shape
    assert np.array_equal(res.view(np.int64), g["residual"].view(np.int64)), np.abs(res - g["residual"]).max()
    assert np.array_equal(its, g["ksp"][:, 1].astype(np.int32))
    for nm in ("U", "V", "W", "P", "T", "R"):
        x = o.get(nm)
        assert np.linalg.norm(x) == g[nm + "_norm"] and np.sum(x) == g[nm + "_sum"], nm
    o.close()


def test_pow15_differs_from_libm_by_one_ulp_at_most():
    """TE^1.5 (the wall function's pow) in the two oracle modes: the once-rounded value the GPU
    computes and the C library's, on the k-epsilon channel fixture; the fields after its six
    iterations stay within relative 1e-12."""
    param = os.path.join(GOLDEN, "channel_tiny", "param.in")
    a, b = po.OracleCase(param), po.OracleCase(param)
    b.set_libm_pow(True)
    for o in (a, b):
        for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
            o.set_ksp(w, po.PC_JACOBI)
        o.iterate(6)
    for nm in ("U", "V", "W", "P", "TE", "ED"):
        x, y = a.get(nm), b.get(nm)
        assert np.linalg.norm(x - y) <= 1e-12 * np.linalg.norm(y), nm


@pytest.mark.skipif(not os.path.isdir(os.environ.get("REF", "/root/reference")) or shutil.which("make") is None,
                    reason="the reference tree is not on this machine")
def test_reference_build_reproduces_fixture(tmp_path):
    """Rebuilds oracle/_ref/cycas_ref from the reference's sources and reruns one fixture: the
    committed vectors are what the reference's own code computes."""
    import make_ref_golden as m
    m.build()
    o = m.run_reference(os.path.join(GOLDEN, "channel_tiny"), 6, [])
    g = dict(np.load(os.path.join(GOLDEN, "channel_tiny", "ref_ilu.npz")))
    assert np.array_equal(o["residual"].reshape(-1, 10).view(np.int64), g["residual"].view(np.int64))
    for nm in ("U", "P", "TE", "ED", "face_n", "cell_vol"):
        assert np.array_equal(o[nm].view(np.int64), g[nm].view(np.int64)), nm
