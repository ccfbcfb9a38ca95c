"""CPU tests of the transient / energy / perfect-gas switches of param.in (NS/readparamfile.cpp:76-140)
and of the initial fields they imply (InitFlowField, NS/navier.cpp:588-697): the library's host
reader against the oracle's, no GPU."""
import os

import numpy as np
import pytest

import pyoracle as po
from sysu_cfd_parallel_gb300 import capi, meshgen
from sysu_cfd_parallel_gb300.solver import Case

CASES = {
    "euler": ("cavity", dict(n=4, time=(0.05, 1.0, 20, "Euler"))),
    "dual": ("cavity", dict(n=4, time=(0.01, 0.25, 7, "Dual"))),
    "energy": ("cavity", dict(n=4, energy=True, wall_t=300, lid_t=320)),
    "gas": ("cavity", dict(n=4, density=1, wall_t=300, lid_t=320)),
    "ke_tr": ("channel", dict(nx=6, ny=2, nz=2, time=(0.1, 1.0, 10, "Dual"), energy=True, wall_t=290)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_physics_and_initial_fields_match_oracle(tmp_path, name):
    kind, kw = CASES[name]
    p = meshgen.write_case(str(tmp_path / name), kind, **kw)
    c = Case(p)
    ph = po.OracleCase(p).physics()
    assert c.steady == ph["steady"] and c.solve_energy == ph["energy"] and c.density_model == ph["density"]
    assert c.max_step == ph["max_step"]
    if not c.steady:
        assert (c.time_scheme, c.max_outer, c.dt, c.total_time) == (ph["time_scheme"], ph["max_outer"], ph["dt"],
                                                                    ph["total_time"])
    o = po.OracleCase(p)
    for nm in ("U", "V", "W", "P", "R", "T", "VisLam", "VisTur"):
        assert np.array_equal(c.get_field(nm).view(np.int64), o.get(nm).view(np.int64)), nm


def test_gas_density_from_the_state_equation(tmp_path):
    p = meshgen.write_case(str(tmp_path / "g"), "cavity", n=3, density=1, wall_t=300, lid_t=320)
    c = Case(p)
    cp = 1006.
    cv = cp / 1.4
    want = (0. + 1.01325e5) / ((cp - cv) * c.get_field("T"))
    assert np.array_equal(c.get_field("R"), want)
    assert c.solve_energy  # DensityModel 1 switches the energy equation on (readparamfile.cpp:337-338)


@pytest.mark.parametrize("line,msg", [("transient,0.1,1.0,5,Crank", "time scheme"),
                                      ("transient,0.1,1.0,Euler", "3 parameters")])
def test_bad_transient_lines(tmp_path, line, msg):
    p = meshgen.write_case(str(tmp_path / "c"), "cavity", n=3)
    text = open(p).read().replace("steady,200,1e-300", line)
    open(p, "w").write(text)
    with pytest.raises(capi.CycasError) as e:
        Case(p)
    assert msg in str(e.value)


def test_server_refuses_non_steady_requests(tmp_path):
    from sysu_cfd_parallel_gb300.solver import Server

    srv = Server(hbm_budget_gb=1.0)
    steady = meshgen.write_case(str(tmp_path / "s"), "cavity", n=3)
    assert srv.submit(steady) >= 1
    for name, kw in (("t", dict(time=(0.1, 1.0, 5, "Euler"))), ("e", dict(energy=True, wall_t=300)),
                     ("g", dict(density=1, wall_t=300))):
        p = meshgen.write_case(str(tmp_path / name), "cavity", n=3, **kw)
        with pytest.raises(capi.CycasError) as e:
            srv.submit(p)
        assert e.value.code == capi.CYCAS_ERR_UNSUPPORTED and "steady" in str(e.value)
    srv.close()
