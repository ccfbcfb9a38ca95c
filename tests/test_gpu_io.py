"""Result files written from device fields (cycas_write_tecplot / _data / _backup, cycas_read_backup).

Each file must equal, byte for byte, the oracle's rendering of the same fields read back through
cycas_get_field: the files then say exactly what the device holds, in the reference's layout.
NSSolve must write them at the reference's cadence, a batch's case must write the file the case
writes alone when its fields are the same, and a backup must restart a solve at the values the
file holds.
"""
import os

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi, results
from sysu_cfd_parallel_gb300.solver import Batch, Case, NavierStokesSolver, batch_options

pytestmark = pytest.mark.gpu

FIELDS = ("P", "U", "V", "W", "R", "T", "VisLam", "VisTur", "TE", "ED")


def _fields(s, k=None):
    return {nm: (s.get(nm) if k is None else s.case_field(nm, k)) for nm in FIELDS}


def _mesh(param):
    o = po.OracleCase(param)
    return o.get("vert"), o.geti("cell_vertices")


@pytest.mark.parametrize("name", ["cavity8j", "channel_tiny"])
def test_result_files_match_oracle_rendering(cases, tmp_path, name):
    p = cases(name)
    c = Case(p)
    s = NavierStokesSolver(c)
    s.iterate(3)
    f = _fields(s)
    vert, cv = _mesh(p)
    s.Output2Tecplot(str(tmp_path / "res0000.dat"))
    s.Output2TecplotBinary(str(tmp_path / "data"))
    s.WriteBackupFile(str(tmp_path / "res.sav"))
    assert (tmp_path / "res0000.dat").read_bytes() == po.tecplot_text(vert, cv, f, c.turb_model).encode()
    assert (tmp_path / "data").read_bytes() == po.data_bytes(f, c.turb_model)
    assert (tmp_path / "res.sav").read_bytes() == po.backup_text(f, c.turb_model).encode()
    # readers
    t = results.read_tecplot(str(tmp_path / "res0000.dat"))
    assert np.array_equal(t["conn"], cv.reshape(-1, 8) + 1)
    np.testing.assert_allclose(t["u"], f["U"], atol=1e-5)
    d, = results.read_data(str(tmp_path / "data"), [c.ncel])
    assert d.shape[0] == (8 if c.turb_model == 1 else 6)
    assert np.array_equal(d[1], f["U"]) and np.array_equal(d[0], f["P"])


def test_backup_round_trip_restarts_at_file_values(cases, tmp_path):
    p = cases("channel_tiny")
    a = NavierStokesSolver(Case(p))
    a.iterate(4)
    a.WriteBackupFile(str(tmp_path / "res.sav"))
    b = NavierStokesSolver(Case(p))
    b.ReadBackupFile(str(tmp_path / "res.sav"))
    fa = _fields(a)
    for nm in ("R", "U", "V", "W", "P", "T", "VisLam", "VisTur", "TE", "ED"):
        want = np.array([float("%g" % x) for x in fa[nm]])
        assert np.array_equal(b.get(nm), want), nm
    b.iterate(2)
    assert np.all(np.isfinite(b.get("U")))


def test_nssolve_writes_at_the_reference_cadence(cases, tmp_path):
    p = cases("cavity8")
    s = NavierStokesSolver(Case(p))
    written = []

    def note(step, rm, res):
        written.append((step, os.path.exists(tmp_path / "tec" / "data")))

    s.NSSolve(max_step=5, residual_steady=0.0, callback=note, output_dir=str(tmp_path), out_binary=True, noutput=3)
    # binary grid before the loop; data after steps 1 and 4; the ASCII result after the loop
    assert (tmp_path / "tec" / "geo").exists() and not (tmp_path / "tec" / "grid.dat").exists()
    assert [w for _, w in written] == [False, True, True, True, True]
    f = _fields(s)
    vert, cv = _mesh(p)
    assert (tmp_path / "tec" / "res0000.dat").read_bytes() == po.tecplot_text(vert, cv, f, 0).encode()
    # the last data and backup files are those of step 4, not of the final step 5
    d, = results.read_data(str(tmp_path / "tec" / "data"), [s.case.ncel])
    assert not np.array_equal(d[1], f["U"])
    assert (tmp_path / "localGeometryBackup_0" / "res.sav").exists()


def test_batch_case_writes_what_the_case_writes_alone(cases, tmp_path):
    names = ["cavity8", "cavity8j", "cavity4"]
    params = [cases(n) for n in names]
    b = Batch([Case(q) for q in params], batch_options())
    b.iterate(2)
    for k, q in enumerate(params):
        alone = NavierStokesSolver(Case(q), batch_options())
        for nm in FIELDS:
            alone.set(nm, b.case_field(nm, k))
        b.Output2Tecplot(str(tmp_path / f"batch{k}.dat"), k=k)
        alone.Output2Tecplot(str(tmp_path / f"alone{k}.dat"))
        b.Output2TecplotBinary(str(tmp_path / f"batch{k}.bin"), k=k)
        alone.Output2TecplotBinary(str(tmp_path / f"alone{k}.bin"))
        assert (tmp_path / f"batch{k}.dat").read_bytes() == (tmp_path / f"alone{k}.dat").read_bytes()
        assert (tmp_path / f"batch{k}.bin").read_bytes() == (tmp_path / f"alone{k}.bin").read_bytes()
    with pytest.raises(capi.CycasError):
        b.Output2TecplotBinary(str(tmp_path / "x.bin"), k=len(params))
