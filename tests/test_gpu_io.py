"""Result files written from device fields (cycas_write_tecplot / _data / _backup, cycas_read_backup).

Each file must equal, byte for byte, the oracle's rendering of the same fields read back through
cycas_get_field: the files then say exactly what the device holds, in the reference's layout.
NSSolve must write them at the reference's cadence, an asynchronous dump must write the fields of
the step it was started at while later iterations run, a batch's case must write the file the
case writes alone when its fields are the same, and a backup must restart a solve at the values
the file holds.
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


@pytest.mark.parametrize("async_output", [False, True])
def test_nssolve_writes_at_the_reference_cadence(cases, tmp_path, async_output):
    p = cases("cavity8")
    s = NavierStokesSolver(Case(p))
    seen = {}

    def note(step, rm, res):
        seen[step] = (s.get("U"), os.path.exists(tmp_path / "tec" / "data"))

    s.NSSolve(max_step=5, residual_steady=0.0, callback=note, output_dir=str(tmp_path), out_binary=True, noutput=3,
              async_output=async_output)
    # binary grid before the loop; data and backup after steps 1 and 4; the ASCII result after the loop
    assert (tmp_path / "tec" / "geo").exists() and not (tmp_path / "tec" / "grid.dat").exists()
    if not async_output:
        assert [seen[k][1] for k in range(1, 6)] == [False, True, True, True, True]
    f = _fields(s)
    vert, cv = _mesh(p)
    assert (tmp_path / "tec" / "res0000.dat").read_bytes() == po.tecplot_text(vert, cv, f, 0).encode()
    # the last data and backup files hold step 4's fields, not the final step's
    d, = results.read_data(str(tmp_path / "tec" / "data"), [s.case.ncel])
    assert np.array_equal(d[1], seen[4][0]) and not np.array_equal(d[1], f["U"])
    back = results.read_backup(str(tmp_path / "localGeometryBackup_0" / "res.sav"), s.case.ncel, 0)
    assert np.array_equal(back["U"], np.array([float("%g" % x) for x in seen[4][0]]))


def test_async_dump_snapshots_the_fields_of_its_step(cases, tmp_path):
    p = cases("channel_small")
    c = Case(p)
    s = NavierStokesSolver(c)
    s.set_graph(True)
    s.iterate(2)
    f = _fields(s)
    s.dump_begin(tecplot=str(tmp_path / "a.dat"), data=str(tmp_path / "a.bin"), backup=str(tmp_path / "a.sav"))
    s.iterate(3)  # the dump's copy-out and formatting overlap these iterations
    s.dump_wait()
    vert, cv = _mesh(p)
    assert (tmp_path / "a.dat").read_bytes() == po.tecplot_text(vert, cv, f, 1).encode()
    assert (tmp_path / "a.bin").read_bytes() == po.data_bytes(f, 1)
    assert (tmp_path / "a.sav").read_bytes() == po.backup_text(f, 1).encode()
    # a dump that cannot write reports it at the wait, and the context stays usable
    s.dump_begin(data=str(tmp_path / "missing" / "b.bin"))
    with pytest.raises(capi.CycasError) as e:
        s.dump_wait()
    assert e.value.code == capi.CYCAS_ERR_IO
    s.dump_wait()
    s.iterate(1)


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
        b.dump_begin(tecplot=str(tmp_path / f"dump{k}.dat"), k=k)
        b.dump_wait()
        assert (tmp_path / f"dump{k}.dat").read_bytes() == (tmp_path / f"alone{k}.dat").read_bytes()
    with pytest.raises(capi.CycasError):
        b.Output2TecplotBinary(str(tmp_path / "x.bin"), k=len(params))
