"""CPU tests of the benchmark's host logic: the replica path across ranks (gloo, world size 2),
the algorithmic-byte model, and the reference arm's rank handling."""
import os
import socket

import pytest

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
        m = bench.reduce_max(ms)
        out.put((rank, m, bench.whole_job_rate(1000, 10, world, m)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [150.0, 150.0]
    # two replicas x 1000 cells x 10 iterations in 0.15 s
    assert all(abs(g[2] - 2 * 1000 * 10 / 0.15) < 1e-6 for g in got)


def test_reduce_max_without_process_group():
    assert bench.reduce_max(3.5) == 3.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup = 1, 0

    assert bench.run_reference(A()) is None
    assert capsys.readouterr().out == ""


def test_krylov_byte_model():
    n, nnz = 1000, 7000
    spmv = 12 * nnz + 4 * (n + 1)
    # one GMRES solve of 2 iterations: residual, 2 Arnoldi steps, solution update
    (kind, slot, its, b), = [r for r in bench.krylov_bytes([2, -1, -1, -1], False, n, nnz) if r[1] == 0]
    step = lambda j: spmv + 24 * n + 8 * n * (j + 2) + 8 * n * (j + 1) + 16 * n
    assert b == spmv + 40 * n + step(0) + step(1) + 8 * n * 4
    # CG with an AMG V-cycle of two levels
    levels = ([n, 250], [nnz, 1500])
    vc = bench.vcycle_bytes(levels)
    assert vc == 24 * nnz + 88 * n + 20 * 250 + 8 * 250 * 250 + 16 * 250
    (_, _, _, bc), = [r for r in bench.krylov_bytes([-1, -1, -1, 3], False, n, nnz, levels=levels) if r[0] == "cg"]
    assert bc == (spmv + 40 * n + vc) + 3 * (spmv + 88 * n + vc)


def test_host_replicas_bounded():
    nproc, cores = bench.host_replicas()
    assert 1 <= nproc <= cores
    assert bench.host_replicas(per_replica_gb=1e9)[0] == 1


def test_l2_flush_is_larger_than_l2_and_reports_when_off():
    """The flush writes twice the GB300's 129 MB L2; where its buffer cannot be made (here: no
    GPU) it is off, calling it does nothing, and the line's l2 note says so instead of claiming a
    flush."""
    assert bench.L2_FLUSH_BYTES >= 2 * 129 * 10**6
    f = bench.L2Flush("cuda:0", None)
    assert f.state.startswith("off (")
    f(None)
    note = bench.l2_note(f)
    assert note.startswith("no flush") and "flushed" not in note
    f.state = "on"
    assert bench.l2_note(f).startswith("L2 flushed before every timed solve")
