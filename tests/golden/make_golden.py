"""Regenerates the golden fixtures in this directory from the oracle.

Each case directory holds the reference-format inputs -- param.in and a gmsh v2 ASCII case.msh,
written by ``sysu_cfd_parallel_gb300.meshgen`` with a fixed seed -- and ``golden.npz`` with the
oracle's outputs on them:

* integer topology in the reference's numbering (element sort of RootStructure.cpp:797-816,
  face discovery of geometry.cpp:222-358) and the CSR pattern;
* geometry (CellFaceInfo, geometry.cpp:391-752);
* the fields, residual history and Krylov iteration counts after ``steps`` SIMPLE-C iterations
  (navier.cpp:60-111) with Jacobi-preconditioned GMRES(30) and CG for the pressure correction
  at the reference's tolerances -- or, for the transient cases, after ``steps`` physical time
  steps (outer iterations of each, ``nouter``), with temperature and density.

The reference itself cannot be built (it needs MPI, PETSc, METIS and CGNS), so these vectors
pin the oracle and the GPU path against each other and against regressions, not against an
executed reference run.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CASES = {
    "cavity5j": dict(kind="cavity", n=5, jitter=0.1, seed=7, mu=0.02, steps=50, golden_steps=8),
    "channel_tiny": dict(kind="channel", nx=10, ny=2, nz=2, steps=20, golden_steps=6),
    # transient cases: golden_steps physical time steps of outer iterations
    "cavity5g_dual": dict(kind="cavity", n=5, jitter=0.1, seed=9, density=1, wall_t=300, lid_t=330,
                          time=(0.05, 1.0, 8, "Dual"), golden_steps=3),
    "channel_tiny_tr": dict(kind="channel", nx=10, ny=2, nz=2, time=(0.1, 1.0, 6, "Euler"), energy=True,
                            wall_t=290, golden_steps=3),
}
INT_ARRAYS = ["face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_face", "cell_cell",
              "cell_vertices", "bnd_face", "bnd_type", "A_rowptr", "A_col"]
GEOMETRY = ["face_x", "face_n", "face_area", "face_lambda", "face_rlencos", "face_xpac", "face_xnac", "cell_vol",
            "cell_x", "bnd_distance"]
FIELDS = ["U", "V", "W", "P", "RUFace"]
FIELDS_KE = ["TE", "ED", "VisTur"]


def write_inputs(name):
    from sysu_cfd_parallel_gb300 import meshgen

    kw = dict(CASES[name])
    kw.pop("golden_steps")
    kind = kw.pop("kind")
    return meshgen.write_case(os.path.join(HERE, name), kind, **kw)


def oracle_outputs(param, steps):
    import pyoracle as po

    o = po.OracleCase(param)
    for w in (po.VELOCITY, po.PRESSURE, po.SCALAR):
        o.set_ksp(w, po.PC_JACOBI, 30)
    out = {nm: o.geti(nm) for nm in INT_ARRAYS}
    out.update({nm: o.get(nm) for nm in GEOMETRY})
    transient = not o.physics()["steady"]
    if transient:
        rs = [o.time_step() for _ in range(steps)]
        out["nouter"] = np.array([r["n"] for r in rs])
        out["resmax"] = np.concatenate([r["resmax"] for r in rs])
        out["residual"] = np.concatenate([r["residual"] for r in rs])
        out["ksp_its"] = np.concatenate([r["ksp_its"] for r in rs])
    else:
        r = o.iterate(steps)
        out["resmax"] = r["resmax"]
        out["residual"] = r["residual"]
        out["ksp_its"] = r["ksp_its"]
    for nm in FIELDS + (FIELDS_KE if o.turb == 1 else []) + (["T", "R"] if transient else []):
        out[nm] = o.get(nm)
    out["steps"] = np.array(steps)
    return out


def main():
    for name, cfg in CASES.items():
        param = write_inputs(name)
        out = oracle_outputs(param, cfg["golden_steps"])
        np.savez_compressed(os.path.join(HERE, name, "golden.npz"), **out)
        print(name, {k: v.shape for k, v in out.items() if k in ("U", "A_col", "resmax")})


if __name__ == "__main__":
    main()
