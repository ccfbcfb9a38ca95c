"""CPU tests of the mesh and result files in the reference's formats (NS/navierIO.cpp,
NS/RootStructure.cpp).

The block layout of the Tecplot writer is pinned by known answers written out by hand from
OutArray2File (navierIO.cpp:2-17); the oracle's Python renderings are checked against those; the
library's grid writers (host code, no GPU) are then compared byte for byte with the oracle's
renderings of the oracle's own mesh, restart files written by the oracle are read back by the
library's case loader, and the compressed binary mesh loads to the same topology as the ASCII one.
"""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi, results
from sysu_cfd_parallel_gb300.solver import Case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def test_block_known_answers():
    # "%19.5f " per value, a line break after every fifth, one after the block
    assert po._block([1.0]) == "            1.00000 \n"
    five = po._block([1, 2, 3, 4, 5])
    assert five == "".join("%19.5f " % v for v in (1, 2, 3, 4, 5)) + "\n\n"
    six = po._block([1, 2, 3, 4, 5, -0.5])
    assert six.splitlines() == ["".join("%19.5f " % v for v in (1, 2, 3, 4, 5)), "           -0.50000 "]
    # rounding to five decimals is the C library's correctly rounded one
    assert po._block([0.000005, 2.675e-5, 123456.123456]) == (
        "            0.00001             0.00003        123456.12346 \n")
    # wider than the 20-character stride: the following value overwrites the tail
    assert po._block([3e13, 1.0]) == "30000000000000.00000            1.00000 \n"
    assert po._block([1.0, 3e13]) == "            1.00000 30000000000000.00000 \n"
    assert po._block([]) == "\n"


def test_tecplot_header_and_zone():
    vert = np.arange(24, dtype=float).reshape(8, 3)
    cv = np.arange(8, dtype=np.int32)
    f = {k: np.array([1.5]) for k in ("P", "U", "V", "W", "R", "T", "VisLam", "VisTur", "TE", "ED")}
    lam = po.tecplot_text(vert, cv, f, 0).split("\n")
    assert lam[0] == 'variables= "x", "y", "z", "p", "u", "v", "w", "ro", "T","Ma","mu" '
    assert lam[1] == ("ZONE N=8, E=1, VARLOCATION=([1-3]=NODAL,[4-11]=CELLCENTERED) DATAPACKING=BLOCK, "
                      "ZONETYPE=FEBRICK")
    ke = po.tecplot_text(vert, cv, f, 1).split("\n")
    assert ke[0].endswith('"mu" "te", "ed"') and "[4-13]" in ke[1]
    # Ma = |u| with constant density, mu = VisLam + VisTur
    text = po.tecplot_text(vert, cv, f, 0)
    assert "%19.5f " % np.sqrt(3 * 1.5 ** 2) in text and "%19.5f " % 3.0 in text
    assert text.endswith("1 2 3 4 5 6 7 8\n ")


def _oracle_mesh(param):
    o = po.OracleCase(param)
    return o, o.get("vert"), o.geti("cell_vertices")


@pytest.mark.parametrize("name", ["cavity5j", "channel_tiny"])
def test_library_grid_files_match_oracle(tmp_path, name):
    param = os.path.join(GOLDEN, name, "param.in")
    o, vert, cv = _oracle_mesh(param)
    c = Case(param)
    assert np.array_equal(c.get_field("vert"), vert)
    c.OutputGrid(str(tmp_path / "grid.dat"))
    c.OutputGridBinary(str(tmp_path / "geo"))
    assert (tmp_path / "grid.dat").read_bytes() == po.grid_text(vert, cv).encode()
    assert (tmp_path / "geo").read_bytes() == po.geo_bytes(vert, cv)
    (v2, conn), = results.read_geo(str(tmp_path / "geo"))
    assert np.array_equal(v2, vert.reshape(-1, 3)) and np.array_equal(conn, cv.reshape(-1, 8) + 1)


def test_grid_write_to_missing_directory_fails(tmp_path):
    c = Case(os.path.join(GOLDEN, "cavity5j", "param.in"))
    with pytest.raises(capi.CycasError) as e:
        c.OutputGrid(str(tmp_path / "no_such_dir" / "grid.dat"))
    assert e.value.code == capi.CYCAS_ERR_IO


def _restart_copy(tmp_path, name, fields, turb):
    d = tmp_path / name
    shutil.copytree(os.path.join(GOLDEN, name), d, ignore=shutil.ignore_patterns("*.npz"))
    lines = [ln for ln in (d / "param.in").read_text().splitlines() if not ln.startswith("restart")]
    (d / "param.in").write_text("\n".join(lines + ["restart,yes"]) + "\n")
    if fields is not None:
        (d / "res.sav").write_text(po.backup_text(fields, turb))
    return str(d / "param.in")


@pytest.mark.parametrize("name", ["cavity5j", "channel_tiny"])
def test_restart_reads_backup_beside_param(tmp_path, name):
    base = Case(os.path.join(GOLDEN, name, "param.in"))
    turb = base.turb_model
    rng = np.random.default_rng(11)
    f = {k: rng.standard_normal(base.ncel) * 10.0 ** rng.integers(-8, 6)
         for k in ("R", "U", "V", "W", "P", "T", "VisLam", "VisTur", "TE", "ED")}
    c = Case(_restart_copy(tmp_path, name, f, turb))
    assert c.restart
    back = results.read_backup(os.path.join(os.path.dirname(c.param_path), "res.sav"), c.ncel, turb)
    names = ["R", "U", "V", "W", "P", "T", "VisLam"] + (["VisTur", "TE", "ED"] if turb == 1 else [])
    for k in names:
        want = np.array([float("%g" % x) for x in f[k]])
        assert np.array_equal(c.get_field(k), want), k
        assert np.array_equal(back[k], want), k
    if turb != 1:
        assert not np.any(c.get_field("VisTur"))


def test_restart_without_backup_fails(tmp_path):
    with pytest.raises(capi.CycasError) as e:
        Case(_restart_copy(tmp_path, "cavity5j", None, 0))
    assert e.value.code == capi.CYCAS_ERR_IO and "res.sav" in str(e.value)


def test_restart_short_backup_fails(tmp_path):
    base = Case(os.path.join(GOLDEN, "cavity5j", "param.in"))
    f = {k: np.ones(base.ncel - 1) for k in ("R", "U", "V", "W", "P", "T", "VisLam")}
    with pytest.raises(capi.CycasError) as e:
        Case(_restart_copy(tmp_path, "cavity5j", f, 0))
    assert e.value.code == capi.CYCAS_ERR_IO


# ---------------------------------------------------------------- compressed binary mesh
INT_ARRAYS = ["face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_face", "cell_cell",
              "cell_vertices", "cell_rid", "bnd_face", "bnd_rid", "bnd_type", "bnd_vertices"]


def _binary_copy(tmp_path, name):
    from sysu_cfd_parallel_gb300 import meshgen

    d = tmp_path / name
    shutil.copytree(os.path.join(GOLDEN, name), d, ignore=shutil.ignore_patterns("*.npz"))
    meshgen.compress_msh(str(d / "case.msh"), str(d / "case.bin"))
    text = (d / "param.in").read_text().replace("gridfile,case.msh", "gridfile,case.bin")
    (d / "param.in").write_text(text)
    return d


@pytest.mark.parametrize("name", ["cavity5j", "channel_tiny"])
def test_binary_mesh_loads_like_ascii(tmp_path, name):
    a = Case(os.path.join(GOLDEN, name, "param.in"))
    d = _binary_copy(tmp_path, name)
    b = Case(str(d / "param.in"), msh_binary=True)
    assert (a.ncel, a.nfac, a.nbnd, a.nvrt) == (b.ncel, b.nfac, b.nbnd, b.nvrt)
    assert np.array_equal(a.get_field("vert").view(np.int64), b.get_field("vert").view(np.int64))
    for nm in INT_ARRAYS:
        assert np.array_equal(a.get_int(nm), b.get_int(nm)), nm
    # record layout: int64 count, then 28-byte vertex records
    raw = (d / "case.bin").read_bytes()
    assert int(np.frombuffer(raw, dtype="<i8", count=1)[0]) >= a.nvrt


def test_binary_mesh_errors(tmp_path):
    d = _binary_copy(tmp_path, "cavity5j")
    raw = (d / "case.bin").read_bytes()
    (d / "case.bin").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(capi.CycasError) as e:
        Case(str(d / "param.in"), msh_binary=True)
    assert e.value.code == capi.CYCAS_ERR_MESH and "truncated" in str(e.value)
    # the ASCII file read as binary is refused, not misread
    text = (d / "param.in").read_text().replace("gridfile,case.bin", "gridfile,case.msh")
    (d / "param.in").write_text(text)
    with pytest.raises(capi.CycasError):
        Case(str(d / "param.in"), msh_binary=True)
    with pytest.raises(capi.CycasError):
        capi.check(capi.load().cycas_case_load_ex(str(d / "param.in").encode(), 4, C.byref(C.c_void_p())))
