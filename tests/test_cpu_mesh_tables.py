"""The host mesh tables on the CPU (sysu_cfd_parallel_gb300/csrc/mesh_tables.cpp, unmodified).

tests/mesh_tables_harness.cpp exposes mesh_tables(); this file checks its output:
* the CSR pattern equals the oracle's (pinned bit-exact to the reference build) on the golden
  meshes, hexahedral and tetrahedral;
* pattern, diagonal positions, slots and both per-cell face orders equal a numpy restatement on
  those meshes and on a 69,120-cell hexahedral grid whose face numbers and per-cell face lists are
  shuffled (large enough for the threaded path);
* a malformed face list is reported for the first failing cell in cell order.
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
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if shutil.which(cxx) is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("mt") / "libmt.so")
    subprocess.run([cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-pthread",
                    os.path.join(ROOT, "sysu_cfd_parallel_gb300", "csrc", "mesh_tables.cpp"),
                    os.path.join(HERE, "mesh_tables_harness.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    ip = C.POINTER(C.c_int)
    L.mt_build.argtypes = [C.c_int, C.c_int, ip, ip, ip, ip, C.POINTER(C.c_long)]
    L.mt_get.argtypes = [C.c_char_p, ip, C.c_long]
    L.mt_error.restype = C.c_char_p
    return L


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _tables(L, nface, cface, f1, f2):
    n, nf = len(nface), len(f1)
    args = [_i32(a) for a in (nface, cface, f1, f2)]
    nnz = C.c_long()
    ip = C.POINTER(C.c_int)
    rc = L.mt_build(n, nf, *[a.ctypes.data_as(ip) for a in args], C.byref(nnz))
    if rc != 0:
        return L.mt_error().decode()
    out = {}
    for name, size in (("rowptr", n + 1), ("col", nnz.value), ("diag", n), ("face_sm", 6 * n), ("gface", 6 * n),
                       ("slot", 6 * n)):
        a = np.zeros(size, np.int32)
        assert L.mt_get(name.encode(), a.ctypes.data_as(ip), size) == 0
        out[name] = a
    return out


def _restate(nface, cface, f1, f2):
    """The tables from their definitions (numpy)."""
    n = len(nface)
    cface = np.asarray(cface, dtype=np.int64).reshape(n, 6)
    j = np.arange(6)[None, :]
    used = j < np.asarray(nface)[:, None]
    cells = np.repeat(np.arange(n)[:, None], 6, axis=1)
    fid = np.where(used, cface, 0)
    nbh = np.where(np.asarray(f2)[fid] < 0, -1, np.where(np.asarray(f1)[fid] == cells, np.asarray(f2)[fid],
                                                          np.asarray(f1)[fid]))
    nbh = np.where(used, nbh, -1)
    keys = np.concatenate([np.arange(n, dtype=np.int64) * n + np.arange(n),
                           (cells.astype(np.int64) * n + nbh)[nbh >= 0]])
    keys = np.unique(keys)
    rowptr = np.concatenate([[0], np.cumsum(np.bincount(keys // n, minlength=n))])
    col = keys % n
    diag = np.searchsorted(keys, np.arange(n, dtype=np.int64) * n + np.arange(n))
    slot = np.where(nbh >= 0, np.searchsorted(keys, cells.astype(np.int64) * n + np.maximum(nbh, 0)), -1)
    big = np.iinfo(np.int64).max
    gface = np.sort(np.where(used, cface, big), axis=1)
    gface = np.where(gface == big, -1, gface)
    face_sm = np.where(used, cface, -1)
    return {"rowptr": rowptr, "col": col, "diag": diag, "slot": slot.T.ravel(), "gface": gface.T.ravel(),
            "face_sm": face_sm.T.ravel()}


def _check(got, want):
    assert isinstance(got, dict), got
    for k, v in want.items():
        assert np.array_equal(got[k], v), k


@pytest.mark.parametrize("name", ["cavity5j", "channel_tiny", "cavity5g_dual", "channel_tiny_tr"])
def test_golden_meshes_match_the_oracle(lib, name):
    o = po.OracleCase(os.path.join(GOLDEN, name, "param.in"))
    topo = [o.geti(k) for k in ("cell_nface", "cell_face", "face_cell1", "face_cell2")]
    got = _tables(lib, *topo)
    assert np.array_equal(got["rowptr"], o.geti("A_rowptr")) and np.array_equal(got["col"], o.geti("A_col"))
    _check(got, _restate(*topo))
    o.close()


def _shuffled_grid(nx, ny, nz, seed):
    """Face topology of an nx x ny x nz hexahedral grid, face numbers and per-cell face lists shuffled."""
    rng = np.random.default_rng(seed)
    cid = np.arange(nx * ny * nz).reshape(nz, ny, nx)
    f1, f2 = [], []
    for axis in range(3):
        pad = [(0, 0)] * 3
        pad[2 - axis] = (1, 1)
        p = np.pad(cid, pad, constant_values=-1)
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[2 - axis] = slice(None, -1)
        b[2 - axis] = slice(1, None)
        lo, hi = p[tuple(a)].ravel(), p[tuple(b)].ravel()
        c1 = np.where(lo >= 0, lo, hi)
        c2 = np.where((lo >= 0) & (hi >= 0), hi, -10)
        f1.append(c1)
        f2.append(c2)
    f1, f2 = np.concatenate(f1), np.concatenate(f2)
    perm = rng.permutation(len(f1))
    f1, f2 = f1[perm], f2[perm]
    n = nx * ny * nz
    nface = np.zeros(n, np.int64)
    cface = -np.ones((n, 6), np.int64)
    for f, (a, b) in enumerate(zip(f1, f2)):
        for c in (a, b) if b >= 0 else (a,):
            cface[c, nface[c]] = f
            nface[c] += 1
    for c in range(n):
        cface[c, :nface[c]] = rng.permutation(cface[c, :nface[c]])
    return nface, cface.ravel(), f1, f2


@pytest.fixture(scope="module")
def grid():
    return _shuffled_grid(48, 40, 36, 11)


def test_shuffled_grid_on_the_threaded_path(lib, grid):
    assert len(grid[0]) >= 1 << 16
    _check(_tables(lib, *grid), _restate(*grid))


def test_first_failing_cell_is_reported(lib, grid):
    nface, cface, f1, f2 = (np.array(a) for a in grid)
    n = len(nface)
    bad = cface.reshape(n, 6).copy()
    far = int(np.flatnonzero((f1 != n - 1) & (f2 != n - 1))[0])
    bad[n - 1, 0] = far  # a face that does not touch the last cell
    assert _tables(lib, nface, bad.ravel(), f1, f2) == "cell_face does not touch its cell"
    bad[100, 1] = len(f1)  # an earlier cell lists a face out of range
    assert _tables(lib, nface, bad.ravel(), f1, f2) == "cell_face out of range"
    nf7 = nface.copy()
    nf7[5] = 7  # and an even earlier one has too many faces
    assert _tables(lib, nf7, bad.ravel(), f1, f2) == "cell_nface out of range"
