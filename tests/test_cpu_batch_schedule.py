"""The team schedule of batched Krylov launches on the CPU
(sysu_cfd_parallel_gb300/csrc/batch_schedule.cpp, unmodified).

A batch's cooperative Krylov launch splits its CTAs into teams: a case with at least
factor * N / G of the batch's N rows gets a team of its own, the smaller cases share single-CTA
teams (largest first onto the least loaded one).  On random batches (equal, uniform and
heavy-tailed case sizes; 1 to 600 cases; 1 to 320 CTAs; the row-share factors the autotuner tries
and others) every schedule must be well formed -- every case in exactly one team, at most G CTAs,
CTA ranks and team offsets consistent -- and follow its rules: an own team has at most
rows / (factor N / G) CTAs and holds one case, a case below the share has no own team, the
shared teams list their cases in ascending order and are balanced as the largest-first greedy
rule guarantees.  Includes the batches that once left no CTA for the smaller cases (more cases
above the share than CTAs, e.g. 200 equal cases on 152 CTAs at factor 0.5).
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
NAMES = ["cta_team", "cta_rank", "team_size", "team_cta0", "team_case0", "case_list"]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if shutil.which(cxx) is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("bs") / "libbs.so")
    subprocess.run([cxx, "-std=c++17", "-O2", "-shared", "-fPIC",
                    os.path.join(ROOT, "sysu_cfd_parallel_gb300", "csrc", "batch_schedule.cpp"),
                    os.path.join(HERE, "batch_schedule_harness.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    ip = C.POINTER(C.c_int)
    L.bs_build.argtypes = [ip, ip, C.c_int, C.c_int, C.c_double]
    L.bs_len.argtypes = [C.c_char_p]
    L.bs_len.restype = C.c_long
    L.bs_get.argtypes = [C.c_char_p, ip, C.c_long]
    L.bs_error.restype = C.c_char_p
    return L


def schedule(L, rows, G, factor):
    hi = np.cumsum(rows).astype(np.int32)
    lo = (hi - np.asarray(rows)).astype(np.int32)
    ip = C.POINTER(C.c_int)
    assert L.bs_build(lo.ctypes.data_as(ip), hi.ctypes.data_as(ip), len(rows), G, factor) == 0, L.bs_error()
    out = {}
    for nm in NAMES:
        n = L.bs_len(nm.encode())
        a = np.zeros(max(n, 1), np.int32)
        assert L.bs_get(nm.encode(), a.ctypes.data_as(ip), n) == 0
        out[nm] = a[:n]
    return out


def check(S, rows, G, factor):
    rows = np.asarray(rows, np.int64)
    nc, N = len(rows), rows.sum()
    target = factor * N / G
    size, cta0, case0, lst = S["team_size"], S["team_cta0"], S["team_case0"], S["case_list"]
    nt = len(size)
    # well formed
    assert np.all(size >= 1) and size.sum() == len(S["cta_team"]) <= G
    assert np.array_equal(cta0, np.concatenate([[0], np.cumsum(size)[:-1]]))
    assert np.array_equal(S["cta_team"], np.repeat(np.arange(nt), size))
    assert np.array_equal(S["cta_rank"], np.concatenate([np.arange(s) for s in size]))
    assert case0[0] == 0 and case0[-1] == nc and len(case0) == nt + 1 and np.all(np.diff(case0) >= 1)
    assert np.array_equal(np.sort(lst), np.arange(nc))
    # the rules
    small_load = []
    for t in range(nt):
        cases = lst[case0[t]:case0[t + 1]]
        if size[t] > 1:
            assert len(cases) == 1
            k = cases[0]
            assert rows[k] >= target and size[t] <= max(1, int(rows[k] / target))
        elif len(cases) == 1 and rows[cases[0]] >= target:
            pass  # an own team of one CTA (or a large case alone in a shared team)
        else:  # a shared team (it may hold large cases that gave up their own team)
            assert np.all(np.diff(cases) > 0)
            small_load.append((rows[cases].sum(), rows[cases].max()))
    for k in range(nc):  # a case below the row share never has a team of several CTAs
        if rows[k] < target:
            t = np.searchsorted(case0, np.flatnonzero(lst == k)[0], side="right") - 1
            assert size[t] == 1
    if len(small_load) > 1:  # largest-first greedy: no shared team exceeds another by more than one case
        loads = np.array([x[0] for x in small_load])
        assert loads.max() - loads.min() <= max(x[1] for x in small_load)


@pytest.mark.parametrize("seed", range(6))
def test_random_batches(lib, seed):
    rng = np.random.default_rng(seed)
    for _ in range(300):
        nc = int(rng.integers(1, 600 if rng.random() < 0.3 else 60))
        kind = rng.integers(3)
        if kind == 0:
            rows = np.full(nc, int(rng.integers(1, 5000)))
        elif kind == 1:
            rows = rng.integers(1, 5000, nc)
        else:
            rows = np.where(rng.random(nc) < 0.1, 200000, rng.integers(1, 3000, nc))
        G = int(rng.integers(1, 321))
        factor = float(rng.choice([0.25, 0.5, 1.0, 2.0, 3.0]))
        check(schedule(lib, rows, G, factor), rows, G, factor)


@pytest.mark.parametrize("nc,G", [(200, 152), (400, 300), (153, 152), (2, 1), (1000, 76)])
def test_more_cases_above_the_share_than_ctas(lib, nc, G):
    rows = np.full(nc, 1000)
    S = schedule(lib, rows, G, 0.5)
    check(S, rows, G, 0.5)
    assert len(S["cta_team"]) <= G


def test_one_large_case_takes_the_grid(lib):
    rows = [500000, 10, 20, 30]
    S = schedule(lib, rows, 152, 1.0)
    check(S, rows, 152, 1.0)
    big = S["team_size"][0]
    assert S["case_list"][0] == 0 and big == 151  # every CTA but the one the small cases share
