"""GPU path (through the C ABI) against the committed golden fixtures of tests/golden/.

Geometry and the CSR pattern are bit-exact; fields after the fixture's SIMPLE iterations (or,
for the transient fixtures, its time steps, with the same number of outer iterations in each)
agree to relative L2 1e-8, residual histories to 1e-6, Krylov iteration counts within one.
"""
import os

import numpy as np
import pytest

from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import Case, NavierStokesSolver

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GEOMETRY = ["face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "face_xpac", "face_xnac", "cell_vol",
            "cell_x", "bnd_distance"]


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


@pytest.mark.parametrize("name", ["cavity5j", "channel_tiny", "cavity5g_dual", "channel_tiny_tr"])
def test_gpu_matches_golden(name):
    param = os.path.join(GOLDEN, name, "param.in")
    g = dict(np.load(os.path.join(GOLDEN, name, "golden.npz")))
    case = Case(param)
    s = NavierStokesSolver(case, capi.default_options(pc=capi.PC_JACOBI))
    for nm in GEOMETRY:
        a = s.get(nm)
        assert np.array_equal(a.view(np.int64), g[nm].view(np.int64)), f"{nm}: max |diff| {np.abs(a - g[nm]).max()}"
    assert np.array_equal(s.get_int("A_rowptr"), g["A_rowptr"])
    assert np.array_equal(s.get_int("A_col"), g["A_col"])
    steps = int(g["steps"])
    transient = "nouter" in g
    if transient:  # physical time steps of outer iterations
        rs = [s.time_step() for _ in range(steps)]
        assert [x["n"] for x in rs] == list(g["nouter"])
        r = {"ksp_its": np.concatenate([x["ksp_its"] for x in rs]), "resmax": np.concatenate([x["resmax"] for x in rs])}
    else:
        r = s.iterate(steps)
    assert np.all(np.abs(r["ksp_its"] - g["ksp_its"]) <= 1), (r["ksp_its"], g["ksp_its"])
    np.testing.assert_allclose(r["resmax"], g["resmax"], rtol=1e-6)
    fields = ["U", "V", "W", "P", "RUFace"] + (["TE", "ED", "VisTur"] if case.turb_model == 1 else [])
    fields += ["T", "R"] if transient else []
    for nm in fields:
        err = _rel_l2(s.get(nm), g[nm])
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"


@pytest.mark.parametrize("name", ["cavity5j", "channel_tiny", "cavity5g_dual", "channel_tiny_tr"])
def test_gpu_matches_reference_build(name):
    """Against the vectors the reference's own sources wrote (ref_jacobi.npz, from
    tests/golden/make_ref_golden.py): geometry bit-exact, the residual of every outer iteration to
    relative 1e-6, fields to relative L2 1e-8, Krylov counts within one."""
    param = os.path.join(GOLDEN, name, "param.in")
    g = dict(np.load(os.path.join(GOLDEN, name, "ref_jacobi.npz")))
    case = Case(param)
    s = NavierStokesSolver(case, capi.default_options(pc=capi.PC_JACOBI))
    for nm in ("face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "cell_vol", "cell_x", "bnd_distance"):
        assert np.array_equal(s.get(nm).view(np.int64), g[nm].view(np.int64)), nm
    interior = g["face_cell2"] >= 0
    for nm in ("face_xpac", "face_xnac"):  # the reference leaves boundary faces at DBL_MAX
        a = s.get(nm).reshape(-1, 3)[interior]
        assert np.array_equal(a.view(np.int64), g[nm].reshape(-1, 3)[interior].view(np.int64)), nm
    steps = int(g["steps"])
    if not case.steady:
        rs = [s.time_step() for _ in range(steps)]
        res = np.concatenate([x["residual"] for x in rs])
        its = np.concatenate([x["ksp_its"] for x in rs])
    else:
        r = s.iterate(steps)
        res, its = r["residual"], r["ksp_its"]
    np.testing.assert_allclose(res, g["residual"], rtol=1e-6, atol=1e-300)
    its = its[its >= 0]
    assert its.shape == g["ksp"][:, 1].shape
    assert np.all(np.abs(its - g["ksp"][:, 1]) <= 1)
    fields = ["U", "V", "W", "P", "RUFace"] + (["TE", "ED", "VisTur"] if case.turb_model == 1 else [])
    fields += ["T", "R"] if not case.steady else []
    for nm in fields:
        err = _rel_l2(s.get(nm), g[nm])
        assert err < 1e-8, f"{nm}: relative L2 {err:.3e}"
    s.close()
