"""Batches (cycas_batch_*): every case advanced in a batch gives the result it gives alone.

Assembly is per cell and per face, so a case's matrices and fields in the union mesh are those
of the case alone; its Krylov solves run on a team of CTAs of their own, whose inner products
sum in a different order than a whole-grid solve.  With every solve converged tightly (rtol
1e-12) the two runs must agree like two runs of the same algorithm: geometry bit-exact, fields
to relative L2 1e-8, residual histories to 1e-6, Krylov iteration counts within one.  At the
reference's own tolerances (pressure rtol 1e-6) a different summation order moves the Krylov
iterates by up to the solver tolerance, so there the bar is relative L2 1e-5.
"""
import numpy as np
import pytest

from sysu_cfd_parallel_gb300.solver import Batch, Case, NavierStokesSolver, batch_options

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    s = np.linalg.norm(b)
    return np.linalg.norm(a - b) / s if s > 0 else np.linalg.norm(a - b)


def _opts(rtol):
    o = batch_options()
    for k in range(3):
        o.ksp[k].rtol = rtol
    return o


def _alone(param, steps, rtol):
    s = NavierStokesSolver(Case(param), _opts(rtol))
    r = s.iterate(steps)
    return s, r


@pytest.mark.parametrize("names,steps", [
    (["cavity4", "cavity8", "cavity8j", "cavity12"], 6),   # small cases: single-CTA teams
    (["cavity36", "cavity8", "cavity4"], 3),                # one multi-CTA team + small ones
    (["channel_tiny", "channel_small"], 4),                 # k-epsilon with outlets
])
def test_batch_matches_cases_alone(cases, names, steps):
    params = [cases(n) for n in names]
    b = Batch([Case(p) for p in params], _opts(1e-12))
    rb = b.iterate(steps)
    turb = b.case.turb_model == 1
    for c, p in enumerate(params):
        s, r = _alone(p, steps, 1e-12)
        for nm in ("cell_vol", "cell_x"):
            a = b.get(nm)
            lo, hi = b.cell0[c], b.cell0[c + 1]
            a = a[3 * lo:3 * hi] if nm == "cell_x" else a[lo:hi]
            assert np.array_equal(a.view(np.int64), s.get(nm).view(np.int64)), nm
        assert np.array_equal(b.case_field("bnd_distance", c).view(np.int64), s.get("bnd_distance").view(np.int64))
        its_b = rb["ksp_its"][:, c, :]
        assert np.all(np.abs(its_b - r["ksp_its"]) <= 1), (names[c], its_b, r["ksp_its"])
        np.testing.assert_allclose(rb["resmax"][:, c], r["resmax"], rtol=1e-6)
        for nm in ["U", "V", "W", "P"] + (["TE", "ED"] if turb else []):
            err = _rel_l2(b.case_field(nm, c), s.get(nm))
            assert err < 1e-8, f"{names[c]} {nm}: relative L2 {err:.3e}"


def test_batch_at_reference_tolerances(cases):
    names = ["cavity8", "cavity8j", "cavity12"]
    params = [cases(n) for n in names]
    b = Batch([Case(p) for p in params])
    rb = b.iterate(8)
    for c, p in enumerate(params):
        s, r = _alone(p, 8, 0.0)
        assert np.all(rb["ksp_reason"][:, c, :4] > 0)
        np.testing.assert_allclose(rb["resmax"][:, c], r["resmax"], rtol=1e-3)
        for nm in ("U", "V", "W", "P"):
            err = _rel_l2(b.case_field(nm, c), s.get(nm))
            assert err < 1e-5, f"{names[c]} {nm}: relative L2 {err:.3e}"


def test_batch_rejects_mixed_physics(cases):
    from sysu_cfd_parallel_gb300 import capi
    with pytest.raises(capi.CycasError):
        Batch([Case(cases("cavity4")), Case(cases("channel_tiny"))])


def test_batch_rebuild_reuses_hierarchies_bit_identically(cases):
    """A case keeps its pressure AMG hierarchy across batches (the server rebuilds a batch at
    every membership change); a batch built from cached hierarchies runs bit-identically to one
    built from fresh cases."""
    names = ["cavity8", "cavity8j", "cavity12"]
    params = [cases(n) for n in names]
    cs = [Case(p) for p in params]
    b1 = Batch(cs, _opts(1e-10))
    r1 = b1.iterate(3)
    b2 = Batch(cs, _opts(1e-10))  # every hierarchy from the cache
    r2 = b2.iterate(3)
    b3 = Batch([Case(params[0]), cs[1], Case(params[2])], _opts(1e-10))  # fresh and cached
    r3 = b3.iterate(3)
    for r in (r2, r3):
        assert np.array_equal(r1["ksp_its"], r["ksp_its"])
    for c in range(3):
        for nm in ("U", "V", "W", "P"):
            a = b1.case_field(nm, c).view(np.int64)
            assert np.array_equal(a, b2.case_field(nm, c).view(np.int64)), (names[c], nm)
            assert np.array_equal(a, b3.case_field(nm, c).view(np.int64)), (names[c], nm)
