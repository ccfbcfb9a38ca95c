"""The union of a batch's cases on the CPU (sysu_cfd_parallel_gb300/csrc/union_mesh.cpp, unmodified).

tests/union_mesh_harness.cpp loads cases with the library's host loader and builds their union;
this file restates the union in numpy from the cases' own arrays -- cells, boundaries and
vertices appended case by case, the boundary faces of all cases first and then all interior
faces, each case's indices shifted by its offsets -- and requires every topology array, every
initial field and the per-case offsets to be equal, on five cases (hexahedral and tetrahedral,
steady and transient; 8,730 cells, enough for the threaded path).  A case that does not number
its boundary faces first is reported.
"""
import ctypes as C
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
CSRC = os.path.join(ROOT, "sysu_cfd_parallel_gb300", "csrc")
sys.path.insert(0, GOLDEN)

INTS = ["face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_rid", "cell_face", "cell_cell",
        "cell_vertices", "bnd_face", "bnd_type", "bnd_rid"]
DBLS = ["vert", "U", "V", "W", "P", "R", "T", "VisLam", "VisTur", "TE", "ED", "BU", "BV", "BW", "BRo", "BTem", "BTE",
        "BED"]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if shutil.which(cxx) is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("un") / "libun.so")
    subprocess.run([cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-pthread",
                    *[os.path.join(CSRC, f) for f in ("host_case.cpp", "result_io.cpp", "union_mesh.cpp")],
                    os.path.join(HERE, "union_mesh_harness.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    L.un_error.restype = C.c_char_p
    L.un_load.argtypes = [C.POINTER(C.c_char_p), C.c_int]
    L.un_build.argtypes = [C.c_int]
    L.un_dims.argtypes = [C.c_int, C.POINTER(C.c_long)]
    L.un_offsets.argtypes = [C.c_int, C.POINTER(C.c_int)]
    L.un_len.argtypes = [C.c_int, C.c_char_p]
    L.un_len.restype = C.c_long
    L.un_geti.argtypes = [C.c_int, C.c_char_p, C.POINTER(C.c_int32), C.c_long]
    L.un_getd.argtypes = [C.c_int, C.c_char_p, C.POINTER(C.c_double), C.c_long]
    return L


def _get(L, k, nm):
    n = L.un_len(k, nm.encode())
    assert n >= 0, nm
    if nm in INTS:
        a = np.zeros(n, np.int32)
        assert L.un_geti(k, nm.encode(), a.ctypes.data_as(C.POINTER(C.c_int32)), n) == 0
    else:
        a = np.zeros(n, np.float64)
        assert L.un_getd(k, nm.encode(), a.ctypes.data_as(C.POINTER(C.c_double)), n) == 0
    return a


def _dims(L, k):
    d = (C.c_long * 4)()
    assert L.un_dims(k, d) == 0
    return list(d)


@pytest.fixture(scope="module")
def loaded(lib, tmp_path_factory):
    from make_ref_golden import write_cavity20
    c20 = os.path.join(write_cavity20(str(tmp_path_factory.mktemp("c20"))), "param.in")
    params = [os.path.join(GOLDEN, "cavity5j", "param.in"), c20, os.path.join(GOLDEN, "channel_tiny", "param.in"),
              os.path.join(GOLDEN, "cavity5g_dual", "param.in"), os.path.join(GOLDEN, "channel_tiny_tr", "param.in")]
    arr = (C.c_char_p * len(params))(*[p.encode() for p in params])
    assert lib.un_load(arr, len(params)) == 0, lib.un_error()
    return len(params)


def _restate(L, nc):
    dims = [_dims(L, k) for k in range(nc)]
    ncel, nfac, nbnd, nvrt = (np.array([d[q] for d in dims]) for q in range(4))
    cell0 = np.concatenate([[0], np.cumsum(ncel)])
    bnd0 = np.concatenate([[0], np.cumsum(nbnd)])
    v0 = np.concatenate([[0], np.cumsum(nvrt)])
    NB = bnd0[-1]
    iface0 = NB + np.concatenate([[0], np.cumsum(nfac - nbnd)])
    NF = NB + (nfac - nbnd).sum()
    out = {nm: [] for nm in INTS + DBLS}
    face = {nm: np.zeros(NF * (4 if nm == "face_vertices" else 1), np.int64)
            for nm in ("face_cell1", "face_cell2", "face_bnd", "face_vertices")}
    for k in range(nc):
        a = {nm: _get(L, k, nm).astype(np.int64) for nm in INTS}

        def fmap(f):
            return np.where(f < nbnd[k], bnd0[k] + f, iface0[k] + f - nbnd[k])
        g = fmap(np.arange(nfac[k]))
        face["face_cell1"][g] = a["face_cell1"] + cell0[k]
        face["face_cell2"][g] = np.where(a["face_cell2"] >= 0, a["face_cell2"] + cell0[k], a["face_cell2"])
        face["face_bnd"][g] = np.where(a["face_bnd"] >= 0, a["face_bnd"] + bnd0[k], a["face_bnd"])
        face["face_vertices"].reshape(-1, 4)[g] = a["face_vertices"].reshape(-1, 4) + v0[k]
        out["cell_nface"].append(a["cell_nface"])
        out["cell_rid"].append(a["cell_rid"])
        out["cell_face"].append(np.where(a["cell_face"] >= 0, fmap(np.maximum(a["cell_face"], 0)), a["cell_face"]))
        out["cell_cell"].append(np.where(a["cell_cell"] >= 0, a["cell_cell"] + cell0[k], a["cell_cell"]))
        out["cell_vertices"].append(a["cell_vertices"] + v0[k])
        out["bnd_face"].append(fmap(a["bnd_face"]))
        out["bnd_type"].append(a["bnd_type"])
        out["bnd_rid"].append(a["bnd_rid"])
        for nm in DBLS:
            out[nm].append(_get(L, k, nm))
    res = {nm: np.concatenate(v) for nm, v in out.items() if v}
    res.update(face)
    return res, (cell0, bnd0, iface0), (cell0[-1], NF, NB, v0[-1])


def test_union_is_the_concatenation_with_renumbered_faces(lib, loaded):
    nc = loaded
    assert lib.un_build(-1) == 0, lib.un_error()
    want, offsets, dims = _restate(lib, nc)
    assert _dims(lib, -1) == [int(x) for x in dims]
    assert sum(_dims(lib, k)[0] * 8 + _dims(lib, k)[1] for k in range(nc)) >= 1 << 16  # threaded
    for kind, w in enumerate(offsets):
        got = (C.c_int * (nc + 1))()
        assert lib.un_offsets(kind, got) == 0
        assert list(got) == [int(x) for x in w], kind
    for nm, w in want.items():
        got = _get(lib, -1, nm)
        assert got.shape == w.shape and np.array_equal(got, w), nm


@pytest.mark.parametrize("broken", [0, 3])
def test_case_without_boundary_faces_first_is_reported(lib, loaded, broken):
    assert lib.un_build(broken) == 1
    assert lib.un_error().decode() == "a batched case does not number its boundary faces first"
