"""cycas_csr_solve_noalloc (device buffers, static scratch) against cycas_csr_solve and the oracle.

Both library entry points run the same persistent GMRES kernel; the no-allocation one only
takes its scratch from a static device array instead of cudaMalloc.  Its results are compared
with the allocating entry point and with the oracle's restatement of PETSc's GMRES, and its
no-allocation property is checked directly: after the warm-up call, further calls leave the
device's free memory unchanged.  Collected last so that it also runs after every other GPU test
has used the device.
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import csr_solve

pytestmark = pytest.mark.gpu

MAX_ROWS = 32768


def _banded(n, seed):
    """Nonsymmetric, diagonally dominant 7-band CSR system."""
    rng = np.random.default_rng(seed)
    offs = np.array([-40, -7, -1, 0, 1, 7, 40])
    rows = np.repeat(np.arange(n), offs.size)
    cols = rows + np.tile(offs, n)
    keep = (cols >= 0) & (cols < n)
    rows, cols = rows[keep], cols[keep]
    vals = np.where(rows == cols, 8.0 + rng.random(rows.size), -rng.random(rows.size))
    rowptr = np.zeros(n + 1, dtype=np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, cols.astype(np.int32), vals, rng.standard_normal(n)


def _noalloc(rowptr, col, val, b, pc, restart, rtol, maxit=1000, x0=None):
    import torch

    dev = torch.device("cuda:0")
    t_rp = torch.from_numpy(rowptr).to(dev)
    t_col = torch.from_numpy(col).to(dev)
    t_val = torch.from_numpy(val).to(dev)
    t_b = torch.from_numpy(b).to(dev)
    guess_zero = x0 is None
    t_x = torch.zeros(b.size, dtype=torch.float64, device=dev) if guess_zero else torch.from_numpy(x0).to(dev)
    stream = torch.cuda.current_stream(dev)
    k = capi.KspOptions(type=capi.KSP_GMRES, restart=restart, pc=pc, rtol=0.0, maxit=0)
    st = capi.SolveStats()
    rc = capi.load().cycas_csr_solve_noalloc(
        b.size, t_rp.data_ptr(), t_col.data_ptr(), t_val.data_ptr(), t_b.data_ptr(), t_x.data_ptr(), C.byref(k),
        rtol, maxit, 1 if guess_zero else 0, C.c_void_p(stream.cuda_stream), C.byref(st))
    return rc, t_x.cpu().numpy(), st


def _rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("pc", [capi.PC_JACOBI, capi.PC_NONE])
def test_noalloc_matches_allocating_solve_on_consecutive_calls(pc):
    # two different systems back to back (the second one at the row limit), then the first again
    systems = [(3000, 1, 20), (MAX_ROWS, 2, 30), (3000, 1, 20)]
    for n, seed, restart in systems:
        rowptr, col, val, b = _banded(n, seed)
        rc, x, st = _noalloc(rowptr, col, val, b, pc, restart, rtol=1e-10)
        assert rc == capi.CYCAS_OK, capi.load().cycas_last_error()
        xr, its_r, reason_r, _ = csr_solve(rowptr, col, val, b, pc=pc, restart=restart, rtol=1e-10)
        assert st.reason > 0 and reason_r > 0
        assert abs(st.its - its_r) <= 1, (st.its, its_r)
        assert _rel_l2(x, xr) < 1e-12
        # the oracle's GMRES(m): classical Gram-Schmidt, left preconditioning, PETSc's test
        xo, its_o, reason_o, _ = po.csr_solve(rowptr, col, val, b, pc={capi.PC_JACOBI: po.PC_JACOBI,
                                                                        capi.PC_NONE: po.PC_NONE}[pc],
                                              restart=restart, rtol=1e-10)
        assert reason_o > 0 and abs(st.its - its_o) <= 1, (st.its, its_o)
        assert _rel_l2(x, xo) < 1e-12


def test_noalloc_allocates_nothing_after_warm_up():
    """After one warm-up call (which may load the module and place the static array), solves of
    the largest size leave cudaMemGetInfo's free bytes unchanged."""
    import torch

    rowptr, col, val, b = _banded(MAX_ROWS, 6)
    dev = torch.device("cuda:0")
    bufs = [torch.from_numpy(a).to(dev) for a in (rowptr, col, val, b)]
    x = torch.zeros(b.size, dtype=torch.float64, device=dev)
    k = capi.KspOptions(type=capi.KSP_GMRES, restart=30, pc=capi.PC_JACOBI, rtol=0.0, maxit=0)
    st = capi.SolveStats()
    lib = capi.load()
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def call():
        x.zero_()
        return lib.cycas_csr_solve_noalloc(b.size, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(),
                                           bufs[3].data_ptr(), x.data_ptr(), C.byref(k), 1e-10, 1000, 1, stream,
                                           C.byref(st))

    assert call() == capi.CYCAS_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(3):
        assert call() == capi.CYCAS_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)


def test_noalloc_initial_guess():
    rowptr, col, val, b = _banded(5000, 3)
    x0 = np.random.default_rng(4).standard_normal(b.size)
    rc, x, st = _noalloc(rowptr, col, val, b, capi.PC_JACOBI, 30, rtol=1e-10, x0=x0)
    assert rc == capi.CYCAS_OK
    xr, its_r, _, _ = csr_solve(rowptr, col, val, b, x0=x0, pc=capi.PC_JACOBI, restart=30, rtol=1e-10,
                                guess_zero=False)
    assert abs(st.its - its_r) <= 1
    assert _rel_l2(x, xr) < 1e-12


def test_noalloc_rejects_oversize_and_unsupported():
    rowptr, col, val, b = _banded(64, 5)
    lib = capi.load()
    rc, _, _ = _noalloc(rowptr, col, val, b, capi.PC_JACOBI, 33, rtol=1e-8)
    assert rc == capi.CYCAS_ERR_INVALID and b"restart" in lib.cycas_last_error()
    rc, _, _ = _noalloc(rowptr, col, val, b, capi.PC_AMG, 30, rtol=1e-8)
    assert rc == capi.CYCAS_ERR_INVALID
    # a row count above the limit is refused before any device memory is touched
    import torch

    t = torch.zeros(64, dtype=torch.float64, device="cuda:0")
    ti = torch.zeros(65, dtype=torch.int32, device="cuda:0")
    k = capi.KspOptions(type=capi.KSP_GMRES, restart=30, pc=capi.PC_JACOBI, rtol=0.0, maxit=0)
    rc = lib.cycas_csr_solve_noalloc(MAX_ROWS + 1, ti.data_ptr(), ti.data_ptr(), t.data_ptr(), t.data_ptr(),
                                     t.data_ptr(), C.byref(k), 1e-8, 100, 1, None, None)
    assert rc == capi.CYCAS_ERR_INVALID and b"32768" in lib.cycas_last_error()
