"""The request server's host logic on the CPU (sysu_cfd_parallel_gb300/csrc/server.cpp, unmodified).

The server is linked with tests/fake_batch_backend.cpp, a deterministic stand-in for the batch
contexts whose cases each need a set number of SIMPLE iterations (see that file).  With the GPU
out of the loop these tests check what the GPU tests cannot pin down: that under any admission
order, budget, cell cap and rebuild mode (in line or on a worker thread) every request does exactly
the iterations it would do alone, with its state carried across every re-forming of its batch;
that admission is first come, first served and never exceeds the budget or the cap (a request
larger than the budget runs alone); that every result is reported once; that transient requests
are refused; that a failed batch build or state copy is reported and leaks nothing; and that no
case is freed while a build still reads it.
"""
import ctypes as C
import os
import random
import shutil
import subprocess
import time

import pytest

from sysu_cfd_parallel_gb300.capi import Options, RequestResult

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

OK, ERR_ALLOC, ERR_CUDA, ERR_UNSUPPORTED = 0, 5, 4, 9
CONVERGED, FAILED, MAX_ITERS = 1, 2, 3


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = os.environ.get("CXX", "g++")
    if shutil.which(cxx) is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("fake") / "libfakeserver.so")
    subprocess.run([cxx, "-std=c++17", "-O1", "-shared", "-fPIC", "-pthread",
                    os.path.join(ROOT, "sysu_cfd_parallel_gb300", "csrc", "server.cpp"),
                    os.path.join(HERE, "fake_batch_backend.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    L.fake_configure.argtypes = [C.c_int] * 4
    L.fake_counters.argtypes = [C.POINTER(i64)]
    L.cycas_server_create.argtypes = [C.POINTER(Options), dbl, dbl, i32, i32, C.POINTER(vp)]
    L.cycas_server_destroy.argtypes = [vp]
    L.cycas_server_set_max_cells.argtypes = [vp, dbl]
    L.cycas_server_set_async_rebuild.argtypes = [vp, i32]
    L.cycas_server_set_graph.argtypes = [vp, i32]
    L.cycas_server_submit.argtypes = [vp, C.c_char_p, C.POINTER(i64)]
    L.cycas_server_step.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    L.cycas_server_poll.argtypes = [vp, C.POINTER(RequestResult), i32, C.POINTER(i32)]
    L.cycas_server_result_field.argtypes = [vp, i64, C.c_char_p, C.POINTER(dbl), i64]
    L.cycas_server_last_error.argtypes = [vp]
    L.cycas_server_last_error.restype = C.c_char_p
    L.cycas_server_stats.argtypes = [vp, C.POINTER(dbl)]
    L.cycas_case_load.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.cycas_case_free.argtypes = [vp]
    L.cycas_footprint_estimate.argtypes = [vp]
    L.cycas_footprint_estimate.restype = dbl
    return L


def counters(L):
    out = (C.c_int64 * 9)()
    L.fake_counters(out)
    keys = ["live_cases", "live_ctx", "creates", "worker_creates", "overlapped", "largest", "copies",
            "use_after_free", "max_cells"]
    return dict(zip(keys, list(out)))


def footprint(L, spec):
    cs = C.c_void_p()
    assert L.cycas_case_load(spec.encode(), C.byref(cs)) == OK
    f = L.cycas_footprint_estimate(cs)
    L.cycas_case_free(cs)
    return f


class Srv:
    def __init__(self, L, budget, tol=1e-6, max_iters=1000, keep_fields=1, async_rebuild=False, max_cells=0.0):
        self.L = L
        self.h = C.c_void_p()
        assert L.cycas_server_create(None, budget, tol, max_iters, keep_fields, C.byref(self.h)) == OK
        assert L.cycas_server_set_async_rebuild(self.h, int(async_rebuild)) == OK
        assert L.cycas_server_set_graph(self.h, 1) == OK
        if max_cells:
            assert L.cycas_server_set_max_cells(self.h, max_cells) == OK
        self.results = {}

    def submit(self, spec):
        i = C.c_int64()
        rc = self.L.cycas_server_submit(self.h, spec.encode(), C.byref(i))
        return rc, i.value

    def step(self):
        a, q = C.c_int32(), C.c_int32()
        rc = self.L.cycas_server_step(self.h, C.byref(a), C.byref(q))
        if rc == OK:
            self.poll()
        return rc, a.value, q.value

    def poll(self):
        buf = (RequestResult * 64)()
        n = C.c_int32()
        while True:
            assert self.L.cycas_server_poll(self.h, buf, 64, C.byref(n)) == OK
            for r in buf[:n.value]:
                assert r.id not in self.results, "reported twice"
                self.results[r.id] = dict(status=r.status, iterations=r.iterations, ncel=r.ncel, t_admit=r.t_admit,
                                          t_done=r.t_done, t_arrival=r.t_arrival, resmax=r.resmax)
            if n.value < 64:
                return

    def field(self, rid, name, n):
        a = (C.c_double * n)()
        assert self.L.cycas_server_result_field(self.h, rid, name.encode(), a, n) == OK
        return list(a)

    def error(self):
        return self.L.cycas_server_last_error(self.h).decode()

    def close(self):
        self.L.cycas_server_destroy(self.h)


def expected(spec, max_iters):
    kv = dict(p.split("=") for p in spec.split(","))
    conv, nan = int(kv.get("conv", 10)), int(kv.get("nan", 0))
    if nan and nan <= min(conv, max_iters):
        return FAILED, nan
    if conv <= max_iters:
        return CONVERGED, conv
    return MAX_ITERS, max_iters


def peak_held(ids, res, weight):
    """The largest `weight` the admitted-and-unfinished requests held at an admission, or None
    if a request was admitted beside others while `weight` exceeded nothing (see overlap_ok)."""
    peak = 0.0
    for i in ids:
        t = res[i]["t_admit"]
        live = [j for j in ids if res[j]["t_admit"] <= t < res[j]["t_done"]]
        if len(live) > 1:
            peak = max(peak, sum(weight[j] for j in live))
    return peak


def overlap_ok(ids, res, weight, cap):
    """At every admission the admitted-and-unfinished requests hold at most `cap` of `weight`,
    unless the one admitted is alone."""
    return peak_held(ids, res, weight) <= cap * (1 + 1e-12)


def run(srv, arrivals, limit=20000):
    """arrivals: {step: [spec, ...]}; steps until nothing is queued or active."""
    ids, specs = [], {}
    last = max(arrivals)
    for step in range(limit):
        for spec in arrivals.get(step, []):
            rc, i = srv.submit(spec)
            assert rc == OK, srv.error()
            ids.append(i)
            specs[i] = spec
        rc, active, queued = srv.step()
        assert rc == OK, srv.error()
        if step >= last and active == 0 and queued == 0:
            break
    else:
        raise AssertionError("the server did not drain")
    # the emptied batches go at a later step (after a build still in flight, if any)
    for _ in range(5000):
        assert srv.step()[0] == OK
        if counters(srv.L)["live_ctx"] == 0:
            break
        time.sleep(0.001)
    return ids, specs


def workload(seed, n=36):
    rng = random.Random(seed)
    arrivals = {}
    for k in range(n):
        step = 0 if k < n // 3 else rng.randrange(0, 150)
        spec = "cells=%d,turb=%d,conv=%d" % (rng.randrange(100, 5000), rng.randrange(2), rng.randrange(2, 45))
        if rng.random() < 0.1:
            spec += ",nan=%d" % rng.randrange(1, 30)
        arrivals.setdefault(step, []).append(spec)
    return arrivals


@pytest.mark.parametrize("async_rebuild", [False, True])
@pytest.mark.parametrize("max_cells", [0.0, 6000.0])
def test_every_request_does_its_own_iterations(lib, async_rebuild, max_cells):
    lib.fake_configure(3, 200, 0, 0)
    arrivals = workload(7)
    allspecs = [s for v in arrivals.values() for s in v]
    fp = {s: footprint(lib, s) for s in allspecs}
    budget = 0.12 * sum(fp.values())
    max_iters = 40
    srv = Srv(lib, budget, max_iters=max_iters, async_rebuild=async_rebuild, max_cells=max_cells)
    ids, specs = run(srv, arrivals)
    res = srv.results
    assert sorted(res) == sorted(ids)
    for i in ids:
        r, spec = res[i], specs[i]
        st, its = expected(spec, max_iters)
        assert (r["status"], r["iterations"]) == (st, its), (spec, r)
        cells = int(spec.split(",")[0].split("=")[1])
        assert r["ncel"] == cells
        u = srv.field(i, "U", cells)
        assert u[0] == its and u[-1] == its, (spec, u[0])  # the case's own state at retirement
        if st == CONVERGED:
            assert abs(r["resmax"] - 0.9e-6) <= 1e-18
        assert r["t_arrival"] <= r["t_admit"] <= r["t_done"]
    admits = [res[i]["t_admit"] for i in ids]
    assert admits == sorted(admits)  # first come, first served across both classes
    assert overlap_ok(ids, res, {i: fp[specs[i]] for i in ids}, budget)
    cells = {i: res[i]["ncel"] for i in ids}
    if max_cells:
        assert overlap_ok(ids, res, cells, max_cells)
        assert peak_held(ids, res, {i: fp[specs[i]] for i in ids}) < budget  # the cap bound first
    # the limits bound: the requests that arrived together would not all have fit
    assert sum(fp[s] for s in arrivals[0]) > budget
    c = counters(lib)
    assert c["use_after_free"] == 0
    assert c["live_ctx"] == 0  # every batch went once its class emptied
    assert c["copies"] > 0  # batches were re-formed with cases continuing
    if async_rebuild:
        assert c["worker_creates"] > 0 and c["overlapped"] > 0
    else:
        assert c["worker_creates"] == 0 and c["overlapped"] == 0
    stats = (C.c_double * 4)()
    assert lib.cycas_server_stats(srv.h, stats) == OK
    assert stats[1] == c["creates"]
    srv.close()
    assert counters(lib)["live_cases"] == 0


def test_request_larger_than_the_budget_runs_alone(lib):
    lib.fake_configure(0, 0, 0, 0)
    small, big = "cells=200,conv=6", "cells=4000,conv=5"
    budget = 1.5 * footprint(lib, "cells=1000")
    assert footprint(lib, big) > budget
    srv = Srv(lib, budget)
    ids, specs = run(srv, {0: [small, big, small], 3: [small]})
    res = srv.results
    b = ids[1]
    others = [i for i in ids if i != b]
    for i in others:  # nothing else is active while the large request runs
        assert res[i]["t_done"] <= res[b]["t_admit"] or res[i]["t_admit"] >= res[b]["t_done"]
    assert res[ids[2]]["t_admit"] >= res[b]["t_done"]  # and the one behind it waits (arrival order)
    for i in ids:
        assert (res[i]["status"], res[i]["iterations"]) == expected(specs[i], 1000)
    srv.close()
    assert counters(lib)["live_cases"] == 0


def test_transient_request_is_refused(lib):
    lib.fake_configure(0, 0, 0, 0)
    srv = Srv(lib, 1e12)
    rc, _ = srv.submit("cells=100,steady=0")
    assert rc == ERR_UNSUPPORTED and "steady" in srv.error()
    assert counters(lib)["live_cases"] == 0
    srv.close()


@pytest.mark.parametrize("async_rebuild", [False, True])
@pytest.mark.parametrize("fault", ["create", "copy"])
def test_failed_rebuild_is_reported_and_leaks_nothing(lib, async_rebuild, fault):
    # the second batch create (the first re-forming, with the first case continuing) or the first
    # state copy fails
    lib.fake_configure(2, 100, 2 if fault == "create" else 0, 1 if fault == "copy" else 0)
    srv = Srv(lib, 1e12, async_rebuild=async_rebuild)
    assert srv.submit("cells=300,conv=30")[0] == OK
    rc = OK
    for step in range(200):
        if step == 2:
            assert srv.submit("cells=500,conv=30")[0] == OK
        rc = srv.step()[0]
        if rc != OK:
            break
    assert rc == (ERR_ALLOC if fault == "create" else ERR_CUDA)
    assert "injected" in srv.error()
    srv.close()
    c = counters(lib)
    assert c["live_ctx"] == 0 and c["live_cases"] == 0 and c["use_after_free"] == 0, c
