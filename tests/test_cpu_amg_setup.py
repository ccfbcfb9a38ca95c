"""The pressure preconditioner's AMG setup on the CPU (sysu_cfd_parallel_gb300/csrc/amg_setup.cpp,
unmodified).

tests/amg_setup_harness.cpp runs the setup with host memory in place of the device and exposes
the hierarchy; this file checks it against independent restatements (numpy / scipy) for several
cases of one system, as a batch holds them:

* aggregation: every row in exactly one non-empty aggregate, each row of a shared aggregate next
  to another row of it, ptptr/ptrow the inverse of agg, maxagg the largest aggregate, level sizes
  falling to at most 64 rows in at most 12 levels;
* Galerkin: every coarse pattern is that of P^T A P (P piecewise constant on the aggregates), and
  random level-0 values carried down the per-depth sum maps (cptr/csrc) equal scipy's P^T A P at
  every level of every case;
* the kept index arrays the cycle reads: diagonals, the row of every diagonal entry, and the next
  level's row of every entry's column (aggcol);
* the SELL-32 copy of every shared-memory level: rows by length (longest first, ties in row
  order), slices padded to their first row with the row's own column, real entries in CSR order;
* the shared-memory tail: 16-byte aligned disjoint regions within its bytes and the budget, rows
  below 65536, the tail as long as the budget allows, and the solver's dynamic shared memory =
  the largest tail + the restriction buffer;
* cycles per tail level by case size (or as forced), and the setup's errors: a system coupling two
  cases, an empty case, a cached hierarchy of another case; a cached hierarchy is used as it is.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "sysu_cfd_parallel_gb300", "csrc")


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if base and os.path.isfile(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
        if os.path.isfile(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx, inc = os.environ.get("CXX", "g++"), _cuda_include()
    if shutil.which(cxx) is None or inc is None:
        pytest.skip("no C++ compiler or CUDA headers")
    so = str(tmp_path_factory.mktemp("amg") / "libamgt.so")
    subprocess.run([cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-I", inc, os.path.join(CSRC, "amg_setup.cpp"),
                    os.path.join(HERE, "amg_setup_harness.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.amgt_error.restype = C.c_char_p
    L.amgt_build.argtypes = [C.c_int, ip, ip, dp, C.c_int, ip, ip, C.c_int, C.c_int]
    for f in ("amgt_depth", "amgt_case"):
        getattr(L, f).argtypes = [C.c_int, ip]
    L.amgt_tail_off.argtypes = [C.c_int, C.c_int, ip]
    L.amgt_level.argtypes = [C.c_int, C.c_int, ip]
    L.amgt_depth_int.argtypes = [C.c_int, C.c_char_p, ip, C.c_long]
    L.amgt_level_int.argtypes = [C.c_int, C.c_int, C.c_char_p, ip, C.c_long]
    L.amgt_level_u16.argtypes = [C.c_int, C.c_int, C.c_char_p, C.POINTER(C.c_ushort), C.c_long]
    return L


def _ints(fn, *args, n):
    a = np.zeros(max(n, 1), dtype=np.int32)
    assert fn(*args, a.ctypes.data_as(C.POINTER(C.c_int)), n) == 0, args
    return a[:n]


def _u16(L, c, l, name, n):
    a = np.zeros(max(n, 1), dtype=np.uint16)
    assert L.amgt_level_u16(c, l, name.encode(), a.ctypes.data_as(C.POINTER(C.c_ushort)), n) == 0
    return a[:n].astype(np.int64)


def _view(L):
    """(ncases, depths, dynamic shared memory of the solver kernel)"""
    a = (C.c_int * 3)()
    L.amgt_view(a)
    return list(a)


def _info(fn, *args, k):
    a = (C.c_int * k)()
    assert fn(*args, a) == 0, args
    return list(a)


# ------------------------------------------------------------------ systems
def _grid(nx, ny, nz):
    """Adjacency of an nx x ny x nz hexahedral mesh (face neighbours)."""
    def path(m):
        return sp.diags([np.ones(m - 1), np.ones(m - 1)], [-1, 1], shape=(m, m))
    I = sp.identity
    return (sp.kron(I(nz), sp.kron(I(ny), path(nx))) + sp.kron(I(nz), sp.kron(path(ny), I(nx))) +
            sp.kron(path(nz), I(ny * nx))).tocsr()


def _random_graph(n, extra, seed):
    """A chain through n rows plus `extra` random couplings (an unstructured pattern)."""
    rng = np.random.default_rng(seed)
    r = np.concatenate([np.arange(n - 1), rng.integers(0, n, extra)])
    c = np.concatenate([np.arange(1, n), rng.integers(0, n, extra)])
    keep = r != c
    A = sp.coo_matrix((np.ones(keep.sum()), (r[keep], c[keep])), shape=(n, n)).tocsr()
    A = A + A.T
    A.data[:] = 1.0
    return A


def _system(adjs, salt=0):
    """Block-diagonal pattern of the cases (diagonal included, columns sorted) with symmetric
    strength weights that vary from face to face (ties broken as on a jittered mesh)."""
    A = sp.block_diag(adjs, format="csr")
    A = (A + sp.identity(A.shape[0], format="csr")).tocsr()
    A.sort_indices()
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    a, b = np.minimum(rows, A.indices).astype(np.int64), np.maximum(rows, A.indices).astype(np.int64)
    w = 1.0 + ((a * 7919 + b * 104729 + salt * 15485863) % 1009) / 1009.0
    sizes = [m.shape[0] for m in adjs]
    hi = np.cumsum(sizes).astype(np.int32)
    lo = np.concatenate([[0], hi[:-1]]).astype(np.int32)
    return A.indptr.astype(np.int32), A.indices.astype(np.int32), w, lo, hi


def _build(L, rowptr, col, w, lo, hi, reuse=0, gamma=0):
    ip = C.POINTER(C.c_int)
    rc = L.amgt_build(len(rowptr) - 1, rowptr.ctypes.data_as(ip), col.ctypes.data_as(ip),
                      w.ctypes.data_as(C.POINTER(C.c_double)), len(lo), lo.ctypes.data_as(ip), hi.ctypes.data_as(ip),
                      reuse, gamma)
    return rc, L.amgt_error().decode()


CASES = [_grid(6, 6, 6), _grid(20, 20, 20), _random_graph(3000, 4500, 1), _grid(12, 30, 9), _grid(4, 4, 4),
         _grid(44, 44, 44)]


@pytest.fixture(scope="module")
def system():
    return _system(CASES)


@pytest.fixture
def built(lib, system):
    """The hierarchies of CASES, built afresh for every test (tests build other systems too)."""
    rowptr, col, w, lo, hi = system
    rc, err = _build(lib, rowptr, col, w, lo, hi)
    assert rc == 0, err
    return system


def _const(L):
    a = (C.c_int * 5)()
    L.amgt_constants(a)
    return dict(zip(["max_levels", "coarse_max", "down_buf", "tail_budget", "w_rows"], list(a)))


def _levels(L, c, rowptr, col, lo, hi):
    """Per level of case c: n, nnz, maxagg, nnz_off, sell_len, row_off and the local pattern."""
    nlev = _info(L.amgt_case, c, k=7)[2]
    out = []
    for l in range(nlev):
        n, nnz, maxagg, nnz_off, sell_len, row_off = _info(L.amgt_level, c, l, k=6)
        if l == 0:
            k0 = rowptr[lo[c]]
            rp = rowptr[lo[c]:hi[c] + 1] - k0
            cl = col[k0:rowptr[hi[c]]] - lo[c]
        else:
            rp = _ints(L.amgt_level_int, c, l, b"rowptr", n=n + 1)
            cl = _ints(L.amgt_level_int, c, l, b"col", n=nnz)
        out.append(dict(n=n, nnz=nnz, maxagg=maxagg, nnz_off=nnz_off, sell_len=sell_len, row_off=row_off, rp=rp, cl=cl))
    return out


def _local_agg(L, c, l, lv, nlev, total_rows):
    if l + 1 >= nlev:
        return None
    if l == 0:
        return _ints(L.amgt_level_int, c, 0, b"agg", n=total_rows)[lv["row_off"]:lv["row_off"] + lv["n"]]
    return _ints(L.amgt_level_int, c, l, b"agg", n=lv["n"])


def test_aggregation_and_galerkin_pattern(lib, built):
    rowptr, col, w, lo, hi = built
    K = _const(lib)
    ncases, depths, _ = _view(lib)
    assert ncases == len(CASES)
    for c in range(ncases):
        lvs = _levels(lib, c, rowptr, col, lo, hi)
        nlev = len(lvs)
        assert nlev <= K["max_levels"] and nlev <= depths
        assert lvs[-1]["n"] <= K["coarse_max"]
        for l in range(nlev - 1):
            F, Cl = lvs[l], lvs[l + 1]
            assert Cl["n"] < F["n"]
            agg = _local_agg(lib, c, l, F, nlev, len(rowptr) - 1)
            assert agg.min() >= 0 and agg.max() == Cl["n"] - 1
            sizes = np.bincount(agg, minlength=Cl["n"])
            assert sizes.min() >= 1 and F["maxagg"] == sizes.max()
            ptptr = _ints(lib.amgt_level_int, c, l, b"ptptr", n=Cl["n"] + 1)
            ptrow = _ints(lib.amgt_level_int, c, l, b"ptrow", n=F["n"]) - (lo[c] if l == 0 else 0)
            assert np.array_equal(ptptr, np.concatenate([[0], np.cumsum(sizes)]))
            assert np.array_equal(ptrow, np.argsort(agg, kind="stable"))
            # a row that shares its aggregate has a neighbour in it
            rows = np.repeat(np.arange(F["n"]), np.diff(F["rp"]))
            off = F["cl"] != rows
            has = np.zeros(F["n"], bool)
            has[rows[off & (agg[F["cl"]] == agg[rows])]] = True
            assert np.all(has | (sizes[agg] == 1))
            # coarse pattern = pattern of P^T A P, columns sorted
            A = sp.csr_matrix((np.ones(F["nnz"]), F["cl"], F["rp"]), shape=(F["n"], F["n"]))
            P = sp.csr_matrix((np.ones(F["n"]), (np.arange(F["n"]), agg)), shape=(F["n"], Cl["n"]))
            G = (P.T @ A @ P).tocsr()
            G.sort_indices()
            assert np.array_equal(G.indptr, Cl["rp"]) and np.array_equal(G.indices, Cl["cl"])
        assert lvs[nlev - 1]["maxagg"] == 0


def test_galerkin_values_through_the_depth_maps(lib, built):
    rowptr, col, w, lo, hi = built
    ncases, depths, _ = _view(lib)
    rng = np.random.default_rng(3)
    vals = [rng.uniform(0.5, 2.0, rowptr[-1])]
    for l in range(depths - 1):
        nrows, nnz, nnz_next = _info(lib.amgt_depth, l, k=3)
        cptr = _ints(lib.amgt_depth_int, l, b"cptr", n=nnz_next + 1)
        csrc = _ints(lib.amgt_depth_int, l, b"csrc", n=int(cptr[-1]))
        assert cptr[0] == 0 and np.all(np.diff(cptr) >= 1)
        seg = np.repeat(np.arange(nnz_next), np.diff(cptr))
        # the fine entries of one coarse entry are listed in ascending order, each fine entry once
        assert np.all((np.diff(csrc) > 0) | (np.diff(seg) > 0))
        assert len(np.unique(csrc)) == len(csrc)
        vals.append(np.bincount(seg, weights=vals[l][csrc], minlength=nnz_next))
    for c in range(ncases):
        lvs = _levels(lib, c, rowptr, col, lo, hi)
        for l in range(len(lvs) - 1):
            F, Cl = lvs[l], lvs[l + 1]
            agg = _local_agg(lib, c, l, F, len(lvs), len(rowptr) - 1)
            k0 = rowptr[lo[c]] if l == 0 else F["nnz_off"]
            fv = vals[l][k0:k0 + F["nnz"]]
            A = sp.csr_matrix((fv, F["cl"], F["rp"]), shape=(F["n"], F["n"]))
            P = sp.csr_matrix((np.ones(F["n"]), (np.arange(F["n"]), agg)), shape=(F["n"], Cl["n"]))
            G = (P.T @ A @ P).tocsr()
            G.sort_indices()
            np.testing.assert_allclose(vals[l + 1][Cl["nnz_off"]:Cl["nnz_off"] + Cl["nnz"]], G.data, rtol=1e-12)


def test_diagonals_and_aggcol(lib, built):
    rowptr, col, w, lo, hi = built
    ncases, depths, _ = _view(lib)
    # level 0: the row of every diagonal entry of the system, -1 elsewhere
    rows0 = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    dr0 = _ints(lib.amgt_depth_int, 0, b"diag_row", n=rowptr[-1])
    assert np.array_equal(dr0, np.where(col == rows0, rows0, -1))
    aggcol0 = _ints(lib.amgt_level_int, 0, 0, b"aggcol", n=rowptr[-1])
    drs = {l: _ints(lib.amgt_depth_int, l, b"diag_row", n=_info(lib.amgt_depth, l, k=3)[1]) for l in range(1, depths)}
    for c in range(ncases):
        lvs = _levels(lib, c, rowptr, col, lo, hi)
        nlev = len(lvs)
        for l, F in enumerate(lvs):
            rows = np.repeat(np.arange(F["n"]), np.diff(F["rp"]))
            if l > 0:
                diag = _ints(lib.amgt_level_int, c, l, b"diag", n=F["n"]) - F["nnz_off"]
                assert np.array_equal(F["cl"][diag], np.arange(F["n"]))
                want = np.where(F["cl"] == rows, F["row_off"] + rows, -1)
                assert np.array_equal(drs[l][F["nnz_off"]:F["nnz_off"] + F["nnz"]], want)
            if l + 1 < nlev:
                agg = _local_agg(lib, c, l, F, nlev, len(rowptr) - 1)
                if l == 0:
                    ac = aggcol0[rowptr[lo[c]]:rowptr[hi[c]]]
                else:
                    ac = _ints(lib.amgt_level_int, c, l, b"aggcol", n=F["nnz"])
                assert np.array_equal(ac, agg[F["cl"]])


def _sell_len(rp):
    ln = np.diff(rp)
    order = np.argsort(-ln, kind="stable")
    ns = (len(ln) + 31) // 32
    return int(sum(32 * ln[order[32 * s]] for s in range(ns)))


def test_sell32_copies_of_the_shared_memory_levels(lib, built):
    rowptr, col, w, lo, hi = built
    ncases = _view(lib)[0]
    checked = 0
    for c in range(ncases):
        tail = _info(lib.amgt_case, c, k=7)[4]
        lvs = _levels(lib, c, rowptr, col, lo, hi)
        for l, F in enumerate(lvs):
            if l < tail or l + 1 >= len(lvs):
                assert F["sell_len"] == 0
                continue
            n, rp, cl = F["n"], F["rp"], F["cl"]
            ns = (n + 31) // 32
            ln = np.diff(rp)
            ptr = _ints(lib.amgt_level_int, c, l, b"sell_ptr", n=ns + 1)
            src = _ints(lib.amgt_level_int, c, l, b"sell_src", n=F["sell_len"])
            scol = _u16(lib, c, l, "sell_col", F["sell_len"])
            perm = _u16(lib, c, l, "sell_row", 32 * ns)[:n]
            assert np.array_equal(perm, np.argsort(-ln, kind="stable"))
            assert F["sell_len"] == ptr[-1] == _sell_len(rp)
            seen = np.zeros(F["nnz"], int)
            for s in range(ns):
                width = (ptr[s + 1] - ptr[s]) // 32
                assert ptr[s + 1] - ptr[s] == 32 * width and width == ln[perm[32 * s]]
                for lane in range(32):
                    p = 32 * s + lane
                    e = ptr[s] + 32 * np.arange(width) + lane
                    if p >= n:
                        assert np.all(src[e] == -1)
                        continue
                    i, k = perm[p], np.arange(width)
                    real = k < ln[i]
                    assert np.array_equal(src[e[real]], rp[i] + k[real])
                    assert np.array_equal(scol[e[real]], cl[rp[i] + k[real]])
                    assert np.all(src[e[~real]] == -1) and np.all(scol[e[~real]] == i)
                    seen[src[e[real]]] += 1
            assert np.all(seen == 1)
            checked += 1
    assert checked > 0


def _region_sizes(lv, lv_next, sell_len, last):
    n, ns = lv["n"], (lv["n"] + 31) // 32
    if last:
        return {"inv": 4 * n * n, "R": 4 * n, "X": 4 * n}
    return {"rowptr": 4 * (ns + 1), "col": 2 * sell_len, "val": 4 * sell_len, "perm": 64 * ns, "wdinv": 4 * n,
            "agg": 4 * n, "ptptr": 4 * (lv_next["n"] + 1), "ptrow": 4 * n, "T": 4 * n, "R": 4 * n, "X": 4 * n}


def _a16(b):
    return (b + 15) // 16 * 16


def test_shared_memory_tail_layout(lib, built):
    rowptr, col, w, lo, hi = built
    K = _const(lib)
    ncases, _, smem = _view(lib)
    names = ["rowptr", "col", "val", "wdinv", "agg", "ptptr", "ptrow", "R", "X", "T", "perm"]
    largest = 0
    for c in range(ncases):
        _, _, nlev, _, tail, nbytes, inv = _info(lib.amgt_case, c, k=7)
        lvs = _levels(lib, c, rowptr, col, lo, hi)
        assert nbytes % 16 == 0 and nbytes <= K["tail_budget"]
        regions = []
        for l in range(K["max_levels"]):
            off = dict(zip(names, _info(lib.amgt_tail_off, c, l, k=11)))
            if l < tail or l >= nlev:
                assert all(v == -1 for v in off.values()), (c, l)
                continue
            assert lvs[l]["n"] < 65536
            last = l == nlev - 1
            sizes = _region_sizes(lvs[l], None if last else lvs[l + 1], lvs[l]["sell_len"], last)
            for nm, size in sizes.items():
                o = inv if nm == "inv" else off[nm]
                assert o >= 0 and o % 16 == 0, (c, l, nm)
                regions.append((o, o + size))
            if last:
                assert all(off[nm] == -1 for nm in names if nm not in ("R", "X"))
        regions.sort()
        assert all(a[1] <= b[0] for a, b in zip(regions, regions[1:]))  # disjoint
        assert regions[-1][1] <= nbytes
        # as long as the budget allows: the next level up would not fit (or has 65536 rows or more)
        if tail > 0:
            up = lvs[tail - 1]
            extra = sum(_a16(v) for v in _region_sizes(up, lvs[tail], _sell_len(up["rp"]), False).values())
            assert up["n"] >= 65536 or nbytes + extra > K["tail_budget"]
        largest = max(largest, nbytes)
    assert smem == largest + 4 * K["down_buf"]


def test_cycles_at_the_first_tail_level(lib, built):
    rowptr, col, w, lo, hi = built
    K = _const(lib)
    for c in range(len(CASES)):
        g = _info(lib.amgt_case, c, k=7)[3]
        assert g == (2 if hi[c] - lo[c] >= K["w_rows"] else 1)
    assert any(hi[c] - lo[c] >= K["w_rows"] for c in range(len(CASES)))
    rc, err = _build(lib, rowptr, col, w, lo, hi, gamma=3)
    assert rc == 0, err
    assert all(_info(lib.amgt_case, c, k=7)[3] == 3 for c in range(len(CASES)))


def test_setup_errors_and_cached_hierarchies(lib):
    a, b = _grid(6, 6, 6), _grid(10, 9, 8)
    rowptr, col, w, lo, hi = _system([a, b])
    assert _build(lib, rowptr, col, w, lo, hi)[0] == 0
    first = [_ints(lib.amgt_level_int, 1, l, b"agg", n=_info(lib.amgt_level, 1, l, k=6)[0]) for l in (1, 2)]
    # other strength weights: a fresh build aggregates differently, the cached hierarchies stay
    _, _, w2, _, _ = _system([a, b], salt=5)
    assert _build(lib, rowptr, col, w2, lo, hi, reuse=1)[0] == 0
    again = [_ints(lib.amgt_level_int, 1, l, b"agg", n=_info(lib.amgt_level, 1, l, k=6)[0]) for l in (1, 2)]
    assert all(np.array_equal(x, y) for x, y in zip(first, again))
    assert _build(lib, rowptr, col, w2, lo, hi)[0] == 0
    fresh0 = _ints(lib.amgt_level_int, 1, 0, b"agg", n=len(rowptr) - 1)
    assert _build(lib, rowptr, col, w, lo, hi)[0] == 0
    assert not np.array_equal(fresh0, _ints(lib.amgt_level_int, 1, 0, b"agg", n=len(rowptr) - 1))
    # the cached hierarchies of another pair of cases
    r2, c2, w3, lo2, hi2 = _system([b, a])
    rc, err = _build(lib, r2, c2, w3, lo2, hi2, reuse=1)
    assert rc == 1 and "another case" in err
    # a system whose couplings cross the cases' rows
    g = _grid(8, 8, 8)
    rowptr, col, w, _, _ = _system([g])
    rc, err = _build(lib, rowptr, col, w, np.array([0, 256], np.int32), np.array([256, 512], np.int32))
    assert rc == 1 and "couples two cases" in err
    rc, err = _build(lib, rowptr, col, w, np.array([0, 512], np.int32), np.array([512, 512], np.int32))
    assert rc == 1 and "empty" in err
