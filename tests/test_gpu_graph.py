"""CUDA-graph replay of whole iterations and the batch schedule autotuner.

Every kernel of the path reduces in a fixed order, so replaying the captured iteration must give
bit-identical fields to issuing the same launches one by one.  The autotuner only changes how
CTAs are grouped into teams, which changes the summation order of the Krylov inner products:
after it, cases still match their runs without it to the tolerance of two runs of the same
algorithm at tight solver tolerances.
"""
import numpy as np
import pytest

from sysu_cfd_parallel_gb300 import capi
from sysu_cfd_parallel_gb300.solver import Batch, Case, NavierStokesSolver, batch_options

pytestmark = pytest.mark.gpu


def _bits(a):
    return a.view(np.int64)


@pytest.mark.parametrize("name", ["cavity8j", "channel_small"])
def test_graph_replay_is_bit_identical(cases, name):
    p = cases(name)
    opts = batch_options()
    a = NavierStokesSolver(Case(p), opts)
    b = NavierStokesSolver(Case(p), opts)
    b.set_graph(True)
    ra = a.iterate(5)
    rb = b.iterate(5)
    assert np.array_equal(ra["ksp_its"], rb["ksp_its"])
    for nm in ("U", "V", "W", "P", "TE", "ED", "RUFace"):
        assert np.array_equal(_bits(a.get(nm)), _bits(b.get(nm))), nm


def test_graph_replay_batch(cases):
    params = [cases(n) for n in ("cavity8", "cavity8j", "cavity12")]
    a = Batch([Case(p) for p in params])
    b = Batch([Case(p) for p in params])
    b.set_graph(True)
    ra = a.iterate(4)
    rb = b.iterate(4)
    assert np.array_equal(ra["ksp_its"], rb["ksp_its"])
    for nm in ("U", "V", "W", "P"):
        assert np.array_equal(_bits(a.get(nm)), _bits(b.get(nm))), nm


def test_autotune_keeps_results(cases):
    params = [cases(n) for n in ("cavity36", "cavity8", "cavity4", "cavity12")]
    o = batch_options()
    for k in range(3):
        o.ksp[k].rtol = 1e-12
    a = Batch([Case(p) for p in params], o)
    b = Batch([Case(p) for p in params], o)
    grid, factor, ms = b.autotune(1)
    assert grid >= 1 and factor > 0 and ms > 0
    a.iterate(9)  # the autotuner ran 9 real iterations
    a.iterate(2)
    b.iterate(2)
    for nm in ("U", "V", "W", "P"):
        x, y = b.get(nm), a.get(nm)
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-8, nm
