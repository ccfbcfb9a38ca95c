"""CPU-only tests: the oracle against the golden fixtures and known answers, the library's host
code (param reader, gmsh reader, face builder) against the oracle, and the C ABI's exports.

No GPU is touched: libcycasgpu.so loads without one, and only host entry points are called.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi, meshgen
from sysu_cfd_parallel_gb300.solver import Case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["cavity5j", "channel_tiny", "cavity5g_dual", "channel_tiny_tr"]
HOST_INT = ["face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_face", "cell_cell",
            "cell_vertices", "bnd_face", "bnd_type"]


def _golden(name):
    return os.path.join(GOLDEN, name, "param.in"), dict(np.load(os.path.join(GOLDEN, name, "golden.npz")))


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


# ---------------------------------------------------------------- golden fixtures
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_inputs_regenerate(tmp_path, name):
    """meshgen still writes the committed reference-format inputs byte for byte."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    kw = dict(mg.CASES[name])
    kw.pop("golden_steps")
    kind = kw.pop("kind")
    p = meshgen.write_case(str(tmp_path / name), kind, **kw)
    for fn in ("param.in", "case.msh"):
        with open(os.path.join(os.path.dirname(p), fn), "rb") as a, open(os.path.join(GOLDEN, name, fn), "rb") as b:
            assert a.read() == b.read(), fn


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_golden(name):
    param, g = _golden(name)
    o = po.OracleCase(param)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, po.PC_JACOBI, 30)
    for nm in ("face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_face", "cell_cell",
               "cell_vertices", "bnd_face", "bnd_type", "A_rowptr", "A_col"):
        assert np.array_equal(o.geti(nm), g[nm]), nm
    for nm in ("face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "face_xpac", "face_xnac", "cell_vol",
               "cell_x", "bnd_distance"):
        np.testing.assert_allclose(o.get(nm), g[nm], rtol=1e-14, atol=1e-15, err_msg=nm)
    steps = int(g["steps"])
    if "nouter" in g:  # transient: physical time steps
        rs = [o.time_step() for _ in range(steps)]
        assert [r["n"] for r in rs] == list(g["nouter"])
        r = {"ksp_its": np.concatenate([x["ksp_its"] for x in rs]), "resmax": np.concatenate([x["resmax"] for x in rs])}
    else:
        r = o.iterate(steps)
    assert np.all(np.abs(r["ksp_its"] - g["ksp_its"]) <= 1)
    np.testing.assert_allclose(r["resmax"], g["resmax"], rtol=1e-6)
    extra = ("T", "R") if "nouter" in g else ()
    for nm in ("U", "V", "W", "P", "RUFace") + (("TE", "ED", "VisTur") if o.turb == 1 else ()) + extra:
        assert _rel_l2(o.get(nm), g[nm]) < 1e-8, nm


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_host_loader_matches_golden(name):
    """The library's C++ param/gmsh reader and sort-based face builder reproduce the
    reference's numbering and face discovery order bit for bit."""
    param, g = _golden(name)
    c = Case(param)
    assert (c.ncel, c.nfac, c.nbnd) == (g["cell_nface"].size, g["face_cell1"].size, g["bnd_face"].size)
    assert c.nnz == g["A_col"].size
    for nm in HOST_INT:
        assert np.array_equal(c.get_int(nm), g[nm]), nm


# ---------------------------------------------------------------- host face builder vs oracle
@pytest.mark.parametrize("kind,kw", [
    ("cavity", dict(n=7, jitter=0.12, seed=11)),
    ("cavity", dict(n=6, planar=False)),
    ("channel", dict(nx=20, ny=4, nz=4, seed=5)),
    ("channel", dict(nx=12, ny=3, nz=5, jitter=0.0)),
])
def test_host_face_builder_bit_exact(tmp_path, kind, kw):
    p = meshgen.write_case(str(tmp_path / "c"), kind, steps=5, **kw)
    c = Case(p)
    o = po.OracleCase(p)
    for nm in HOST_INT + ["cell_rid", "bnd_rid", "bnd_vertices"]:
        assert np.array_equal(c.get_int(nm), o.geti(nm)), nm


# ---------------------------------------------------------------- known answers
@pytest.fixture(scope="module")
def cavity6(tmp_path_factory):
    p = meshgen.write_case(str(tmp_path_factory.mktemp("k") / "cav6"), "cavity", n=6, steps=5)
    return po.OracleCase(p)


@pytest.fixture(scope="module")
def channel_j(tmp_path_factory):
    p = meshgen.write_case(str(tmp_path_factory.mktemp("k") / "ch"), "channel", nx=12, ny=3, nz=3, steps=5)
    return po.OracleCase(p)


def test_volumes_sum_to_domain(cavity6, channel_j):
    assert abs(cavity6.get("cell_vol").sum() - 1.0) < 1e-12
    assert abs(channel_j.get("cell_vol").sum() - 10.0) < 1e-11  # 10 x 1 x 1 box
    assert np.all(channel_j.get("cell_vol") > 0)


@pytest.mark.parametrize("which", ["cavity6", "channel_j"])
def test_cells_are_closed(request, which):
    """Face.n is the area vector (|n| = area, geometry.cpp:590-603), oriented from cell1 to
    cell2; summed over a cell's faces with outward signs it vanishes."""
    o = request.getfixturevalue(which)
    n = o.get("face_n").reshape(-1, 3)
    area = o.get("face_area")
    np.testing.assert_allclose(np.linalg.norm(n, axis=1), area, rtol=1e-14)
    c1, c2 = o.geti("face_cell1"), o.geti("face_cell2")
    xf, xc = o.get("face_x").reshape(-1, 3), o.get("cell_x").reshape(-1, 3)
    assert np.all(np.einsum("ij,ij->i", n, xf - xc[c1]) > 0)
    acc = np.zeros((o.ncel, 3))
    np.add.at(acc, c1, n)
    inner = c2 >= 0
    np.add.at(acc, c2[inner], -n[inner])
    assert np.abs(acc).max() < 1e-14 * area.max() * 100


def test_green_gauss_exact_on_linear_field(cavity6):
    """On a uniform hex grid the face value lambda*phi1+(1-lambda)*phi2 of a linear field is its
    value at the face centre, so Green-Gauss (navier_gradient.cpp:12-74) returns the slope."""
    o = cavity6
    a = np.array([0.3, -1.7, 2.5])
    xc = o.get("cell_x").reshape(-1, 3)
    xf = o.get("face_x").reshape(-1, 3)
    bf = o.geti("bnd_face")
    o.set("deltaP", xc @ a + 0.25)
    o.set("BPre", xf[bf] @ a + 0.25)
    o.stage("grad_deltap")
    g = o.get("dPdX").reshape(-1, 3)
    np.testing.assert_allclose(g, np.broadcast_to(a, g.shape), rtol=0, atol=1e-12)


@pytest.mark.parametrize("which", ["cavity6", "channel_j"])
def test_csr_pattern(request, which):
    """Diagonal + one entry per interior-face neighbour, columns ascending (PETSc AIJ), pattern
    symmetric, nnz = Nc + 2 Nfi."""
    o = request.getfixturevalue(which)
    rp, col = o.geti("A_rowptr"), o.geti("A_col")
    nfi = int((o.geti("face_cell2") >= 0).sum())
    assert rp[0] == 0 and rp[-1] == col.size == o.ncel + 2 * nfi
    rows = np.repeat(np.arange(o.ncel), np.diff(rp))
    for i in range(o.ncel):
        seg = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(seg) > 0) and i in seg
    pairs = set(zip(rows.tolist(), col.tolist()))
    assert all((j, i) in pairs for (i, j) in pairs)


@pytest.mark.parametrize("which", ["cavity6", "channel_j"])
def test_pressure_rows_sum_to_zero(request, which):
    """Pressure-correction rows: diagonal -sum(tmp), off-diagonals +tmp, boundary faces skipped
    for constant density (navier_pressure.cpp:99-232), so every row sums to zero and the matrix
    is symmetric; the right-hand side is the cell's mass imbalance."""
    o = request.getfixturevalue(which)
    o.iterate(2)
    o.stage("build_velocity")
    o.stage("ruface2")
    o.stage("build_pressure")
    rp, col, val = o.geti("A_rowptr"), o.geti("A_col"), o.get("Ap_val")
    rows = np.repeat(np.arange(o.ncel), np.diff(rp))
    diag = val[rows == col]
    rs = np.zeros(o.ncel)
    np.add.at(rs, rows, val)
    assert np.all(diag < 0)
    assert np.abs(rs).max() <= 1e-12 * np.abs(diag).max()
    dense = {(int(i), int(j)): v for i, j, v in zip(rows, col, val)}
    assert max(abs(v - dense[(j, i)]) for (i, j), v in dense.items()) <= 1e-14 * np.abs(diag).max()
    # b = sum over the cell's faces of the signed face flux
    ru = o.get("RUFace")
    c1, c2 = o.geti("face_cell1"), o.geti("face_cell2")
    imb = np.zeros(o.ncel)
    np.add.at(imb, c1, ru)
    inner = c2 >= 0
    np.add.at(imb, c2[inner], -ru[inner])
    np.testing.assert_allclose(np.abs(o.get("bp")), np.abs(imb), rtol=1e-10, atol=1e-14)


def test_oracle_krylov_known_answer():
    """GMRES and CG restatements solve a small SPD system to the requested tolerance."""
    n = 50
    main = np.full(n, 4.0); off = np.full(n - 1, -1.0)
    rows = np.concatenate([np.arange(n), np.arange(n - 1), np.arange(1, n)])
    cols = np.concatenate([np.arange(n), np.arange(1, n), np.arange(n - 1)])
    vals = np.concatenate([main, off, off])
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int32)
    x_true = np.sin(np.arange(n))
    A = np.zeros((n, n)); A[rows, cols] = vals
    b = A @ x_true
    for kt in (po.KSP_GMRES, po.KSP_CG):
        for pc in (po.PC_NONE, po.PC_JACOBI, po.PC_ILU0):
            x, its, reason, _ = po.csr_solve(rp, cols, vals, b, rtol=1e-12, pc=pc, ksp_type=kt)
            assert reason > 0 and its > 0
            assert np.abs(x - x_true).max() < 1e-9


# ---------------------------------------------------------------- host input errors
def _write(tmp_path, text, mesh_from=None):
    d = tmp_path / "bad"
    d.mkdir(exist_ok=True)
    if mesh_from:
        (d / "case.msh").write_bytes(open(mesh_from, "rb").read())
    (d / "param.in").write_text(text)
    return str(d / "param.in")


def test_param_errors(tmp_path):
    good = open(os.path.join(GOLDEN, "cavity5j", "param.in")).read()
    mesh = os.path.join(GOLDEN, "cavity5j", "case.msh")
    with pytest.raises(capi.CycasError) as e:
        Case(str(tmp_path / "nope.in"))
    assert e.value.code == capi.CYCAS_ERR_IO
    with pytest.raises(capi.CycasError) as e:
        Case(_write(tmp_path, good + "frobnicate,1\n", mesh))
    assert e.value.code == capi.CYCAS_ERR_INVALID and "no such command" in str(e.value)
    with pytest.raises(capi.CycasError) as e:
        Case(_write(tmp_path, good.replace("bound,1,Hwall,walls,0", "bound,1,Hwall,walls"), mesh))
    assert e.value.code == capi.CYCAS_ERR_INVALID and "wall requires 1 parameter" in str(e.value)
    with pytest.raises(capi.CycasError) as e:
        Case(_write(tmp_path, good.replace("gridfile,case.msh", "gridfile,missing.msh"), mesh))
    assert e.value.code == capi.CYCAS_ERR_IO


def test_mesh_errors(tmp_path):
    good = open(os.path.join(GOLDEN, "cavity5j", "param.in")).read()
    text = open(os.path.join(GOLDEN, "cavity5j", "case.msh")).read()
    d = tmp_path / "m"
    d.mkdir()
    (d / "param.in").write_text(good)
    (d / "case.msh").write_text(text.replace("$Nodes", "$NoNodes"))
    with pytest.raises(capi.CycasError) as e:
        Case(str(d / "param.in"))
    assert e.value.code == capi.CYCAS_ERR_MESH


# ---------------------------------------------------------------- C ABI surface
def _header_functions():
    text = open(os.path.join(ROOT, "include", "cycasgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cycas_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    names = _header_functions()
    assert len(names) >= 20
    lib = C.CDLL(capi.library_path() if os.path.exists(capi.library_path()) else capi.load()._name)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(capi.EXPORTS) == names


@pytest.mark.parametrize("ref", [-1, 8, 1000])
def test_create_rejects_a_reference_cell_outside_the_mesh(ref):
    """The kernels read p' at cellPressureRef: a value outside the mesh is an argument error,
    reported before anything reaches a device (so this runs without one)."""
    L = capi.load()
    mesh = capi.MeshView()
    mesh.ncel, mesh.nfac, mesh.nbnd, mesh.nvrt = 8, 36, 24, 27
    p = capi.Params()
    p.cell_pressure_ref = ref
    ctx = C.c_void_p()
    assert L.cycas_create(C.byref(mesh), C.byref(p), None, C.byref(ctx)) == capi.CYCAS_ERR_INVALID
    assert capi.last_error() == "PressureRef cell out of range" and not ctx.value


def test_header_is_a_plain_c_abi(tmp_path):
    """include/cycasgpu.h compiles as pedantic C99 and C++11, and a C program links the library and
    calls a host entry point through it (no GPU needed for the defaults)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text('#include "cycasgpu.h"\n'
                   "int main(void) { cycas_options o; cycas_options_default(&o);\n"
                   "  return o.ksp[0].restart == 30 && o.ksp[1].restart == 30 ? 0 : 1; }\n")
    inc = os.path.join(ROOT, "include")
    flags = ["-Wall", "-Wextra", "-pedantic", "-Werror", "-I", inc, "-c", str(src)]
    subprocess.run(["gcc", "-std=c99", *flags, "-o", str(tmp_path / "c.o")], check=True)
    subprocess.run(["g++", "-std=c++11", "-x", "c++", *flags, "-o", str(tmp_path / "cxx.o")], check=True)
    lib = capi.library_path() if os.path.exists(capi.library_path()) else capi.load()._name
    exe = str(tmp_path / "abi")
    subprocess.run(["gcc", "-std=c99", "-I", inc, str(src), lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe],
                   check=True)
    assert subprocess.run([exe]).returncode == 0


def test_defaults_follow_reference():
    o = capi.Options()
    capi.load().cycas_options_default(C.byref(o))
    assert [o.ksp[s].type for s in range(3)] in ([capi.KSP_DEFAULT] * 3, [capi.KSP_GMRES, capi.KSP_CG, capi.KSP_GMRES])
    assert all(o.ksp[s].restart == 30 for s in range(3))


def test_mesh_cache_reuses_and_invalidates(tmp_path):
    """The loader parses a mesh file once per version: a second case over the same file gets
    the same arrays with its own parameters, and a rewritten file is parsed again."""
    d = tmp_path / "mc"
    p = meshgen.write_case(str(d), "cavity", n=5, jitter=0.1, seed=3, steps=5)
    a = Case(p)
    text = open(p).read().replace("0.01", "0.05")
    p2 = str(d / "param2.in")
    open(p2, "w").write(text)
    b = Case(p2)
    for nm in HOST_INT + ["cell_rid", "bnd_rid", "bnd_vertices"]:
        assert np.array_equal(a.get_int(nm), b.get_int(nm)), nm
    assert np.array_equal(a.get_field("VisLam") * 5.0, b.get_field("VisLam"))
    meshgen.write_case(str(d), "cavity", n=6, steps=5)  # same path, another mesh
    c = Case(p)
    assert c.ncel == 216 and a.ncel == 125
    o = po.OracleCase(p)
    for nm in HOST_INT:
        assert np.array_equal(c.get_int(nm), o.geti(nm)), nm
