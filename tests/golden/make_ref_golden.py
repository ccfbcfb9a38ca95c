"""Regenerates the fixtures of this directory that come from the reference's own code.

``oracle/refpin`` builds the reference's unmodified solver sources (NS/*.cpp, read where they lie)
against a single-rank stand-in for MPI, PETSc, METIS and CGNS whose Krylov solves are the
oracle's (see oracle/refpin/include/petscksp.h).  ``oracle/_ref/cycas_ref`` then runs the
reference's own start-up sequence and NSSolve on a case and writes what it built and computed.
This script runs it on the committed case inputs and stores, per case and preconditioner,
``ref_<pc>.npz``:

* the integer topology and geometry the reference built (CreateFaces / CellFaceInfo);
* the residual vector NSSolve reduced in every outer iteration (navier.cpp:94);
* every Krylov solve's iteration count and converged reason;
* the fields after the run (for ``cavity20`` only u, v, w and p, besides the residual history
  and the Krylov log).

The cases are those of make_golden.py (run for ``golden_steps`` iterations or time steps) plus
``cavity20``, the plain-method cavity (20^3 hexahedra, Re 100) for its configured 200 iterations
with GMRES(30) rtol 1e-8 on every system (-ksp_type gmres -ksp_rtol 1e-8), as the configuration
runs the reference.  Preconditioners: ``ilu`` (PETSc's default, ILU(0)) and ``jacobi``.

``cavity48/ref_ilu_tight.npz``: the bench's cavity (48^3 hexahedra) for its first 5 SIMPLE
iterations with the reference's own solvers and ILU(0), every system to rtol 1e-10
(-ksp_rtol 1e-10): residual history, Krylov log, and the L2 norm and sum of u, v, w, p (the
fields themselves would be megabytes).

``cavity48/ref_ilu_converged.npz``: the bench's cavity (48^3) run by the reference build to its
own stop test (NSSolve's ResMax < 1e-6, the param's residual) at its own tolerances and ILU(0):
ResMax of every SIMPLE iteration (about 15 minutes on one core; not run by main()).

``batch_cavities/ref_stop.npz``: the cavities of the batched workload (seed 4: n^3 hexahedra with
n uniform in 8..40, jitter 0.1h, mu = 1/Re with Re log-uniform in [10, 1000]) that have at most
40^3 cells (all 256), each run by the reference build to its own stop test (ResMax < 1e-6) with
ILU(0): the SIMPLE iteration at which each stops (about 20 minutes on 8 cores; not run by main()).

``channel_coarse/ref_ilu.npz``: the configured k-epsilon channel's physics on a coarse mesh
(50x5x5 hexahedra split into 6 jittered Kuhn tetrahedra each, 7,500 cells, jitter 0.15h, seed
2026) for its first 10 SIMPLE iterations at the reference's own tolerances and ILU(0): residual
history, Krylov log, and the L2 norm and sum of u, v, w, p, k, epsilon.

``channel_coarse_tr/ref_ilu.npz``: the same mesh run transient (Euler, dt 0.1, at most 6 outer
iterations per step) with the energy equation and 290 K walls, for 3 time steps at the
reference's tolerances and ILU(0): residual history of every outer iteration, Krylov log, and
the L2 norm and sum of u, v, w, p, k, epsilon, T, rho.

``cavity16g_dual/ref_ilu.npz``: a perfect-gas cavity (16^3 hexahedra, jitter 0.1h, walls 300 K,
lid 330 K) with the reference's second-order "Dual" scheme (dt 0.05, at most 8 outer iterations
per step) for 3 time steps at the reference's tolerances and ILU(0): residual history, Krylov
log, and the L2 norm and sum of u, v, w, p, T, rho.

Needs the reference tree (REF, default /root/reference) and g++.  Run from the repository root:
    python tests/golden/make_ref_golden.py
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("REF", "/root/reference")
BINARY = os.path.join(ROOT, "oracle", "_ref", "cycas_ref")

# name -> (golden steps, extra reference options)
RUNS = {
    "cavity5j": (8, []),
    "channel_tiny": (6, []),
    "cavity5g_dual": (3, []),
    "channel_tiny_tr": (3, []),
    "cavity20": (200, ["-ksp_type", "gmres", "-ksp_rtol", "1e-8"]),
}
GEOMETRY_INT = ["face_cell1", "face_cell2", "face_bnd", "face_vertices", "cell_nface", "cell_rid", "cell_face",
                "cell_cell", "cell_vertices", "cell_globalidx", "bnd_face", "bnd_rid", "bnd_vertices"]
GEOMETRY = ["face_x", "face_n", "face_xpac", "face_xnac", "face_area", "face_lambda", "face_rlencos", "cell_vol",
            "cell_x", "bnd_distance", "vert"]
FIELDS = ["U", "V", "W", "P", "R", "T", "VisTur", "RUFace", "deltaP", "Apr", "TE", "ED"]


def build():
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "refpin"), "REF=" + REF], check=True)
    return BINARY


def load_outputs(out):
    d = {}
    with open(os.path.join(out, "manifest.txt")) as f:
        for line in f:
            nm, dt, n = line.split()
            d[nm] = np.fromfile(os.path.join(out, nm + ".bin"), dtype={"f8": np.float64, "i4": np.int32}[dt])
    return d


def run_reference(case_dir, steps, options=()):
    """Runs the reference build on a copy of case_dir; returns its outputs as arrays."""
    with tempfile.TemporaryDirectory() as tmp:
        work = os.path.join(tmp, "case")
        os.makedirs(work)
        for f in ("case.msh", "param.in"):
            shutil.copy(os.path.join(case_dir, f), work)
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        r = subprocess.run([BINARY, work, out, "--iters", str(steps), *options], stdin=subprocess.DEVNULL,
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, env=dict(os.environ, TERM="dumb"))
        if r.returncode != 0:
            raise RuntimeError(r.stdout.decode(errors="replace")[-3000:])
        return load_outputs(out)


def pack(o, steps, options, geometry=True):
    keep = {nm: o[nm] for nm in GEOMETRY_INT + GEOMETRY if nm in o} if geometry else {}
    keep.update({nm: o[nm] for nm in (FIELDS if geometry else ["U", "V", "W", "P"]) if nm in o})
    keep["residual"] = o["residual"].reshape(-1, 10)
    keep["ksp"] = o["ksp"].reshape(-1, 4)
    keep["info"] = o["info"]
    keep["steps"] = np.array(steps)
    keep["options"] = np.array(" ".join(options))
    return keep


def write_cavity20(d):
    """The 20^3 cavity's inputs (uniform mesh, no random numbers: meshgen writes the same bytes
    every time, so only the fixtures are committed)."""
    from sysu_cfd_parallel_gb300 import meshgen
    return os.path.dirname(meshgen.write_case(d, "cavity", n=20, steps=200))


def write_cavity48(d):
    """The bench's cavity inputs (48^3 uniform hexahedra; meshgen writes the same bytes every time)."""
    from sysu_cfd_parallel_gb300 import meshgen
    return os.path.dirname(meshgen.write_case(d, "cavity", n=48, steps=5))


CAVITY48_OPTIONS = ["-ksp_rtol", "1e-10"]
CAVITY48_STEPS = 5


def cavity48_fixture():
    tmp = tempfile.mkdtemp()
    try:
        o = run_reference(write_cavity48(tmp), CAVITY48_STEPS, CAVITY48_OPTIONS)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    keep = {"residual": o["residual"].reshape(-1, 10), "ksp": o["ksp"].reshape(-1, 4), "info": o["info"],
            "steps": np.array(CAVITY48_STEPS), "options": np.array(" ".join(CAVITY48_OPTIONS))}
    for nm in ("U", "V", "W", "P"):
        keep[nm + "_norm"] = np.array(np.linalg.norm(o[nm]))
        keep[nm + "_sum"] = np.array(np.sum(o[nm]))
    os.makedirs(os.path.join(HERE, "cavity48"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "cavity48", "ref_ilu_tight.npz"), **keep)
    print("cavity48 iterations", o["residual"].size // 10, "solves", o["ksp"].size // 4)


def cavity48_converged_fixture():
    """The bench cavity to the reference's own stop test; keeps ResMax of every iteration."""
    from sysu_cfd_parallel_gb300 import meshgen
    tmp = tempfile.mkdtemp()
    try:
        d = os.path.dirname(meshgen.write_case(tmp, "cavity", n=48, steps=3000, residual=1e-6))
        o = run_reference(d, 3000, [])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    res = o["residual"].reshape(-1, 10)
    resmax = np.maximum(res.max(axis=1), 0.0)  # vec_max of localRes, floored at 0 (navier.cpp:94-96)
    os.makedirs(os.path.join(HERE, "cavity48"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "cavity48", "ref_ilu_converged.npz"), resmax=resmax,
                        residual_steady=np.array(1e-6))
    print("cavity48 to the stop test: iterations", len(resmax), "last ResMax", resmax[-1])


BATCH_SEED = 4  # the batched workload's master seed


def batch_cavity_specs():
    """(n, mesh seed, mu) of the batched workload's 256 cavities, in case order."""
    rng = np.random.default_rng(BATCH_SEED)
    ns = rng.integers(8, 41, size=256)
    res = 10.0 ** rng.uniform(1.0, 3.0, size=256)
    return [(int(ns[k]), 1000 + k, float(1.0 / res[k])) for k in range(256)]


def write_batch_cavity(d, n, seed, mu):
    from sysu_cfd_parallel_gb300 import meshgen
    return os.path.dirname(meshgen.write_case(d, "cavity", n=n, jitter=0.1, seed=seed, steps=2000, mu=mu,
                                              residual=1e-6))


def batch_stop_fixture(max_n=40, workers=8):
    """Every case runs as its own reference process; `workers` of them at a time."""
    from concurrent.futures import ThreadPoolExecutor
    specs = batch_cavity_specs()
    rows = [k for k in sorted(range(256), key=lambda k: (specs[k][0], k)) if specs[k][0] <= max_n]

    def one(k):
        tmp = tempfile.mkdtemp()
        try:
            o = run_reference(write_batch_cavity(tmp, *specs[k]), 2000, [])
        finally:
            shutil.rmtree(tmp, ignore_errors=True)
        return o["residual"].size // 10  # NSSolve stopped at ResMax < 1e-6

    with ThreadPoolExecutor(max_workers=workers) as ex:
        stop = list(ex.map(one, rows))
    k = np.array(rows)
    os.makedirs(os.path.join(HERE, "batch_cavities"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "batch_cavities", "ref_stop.npz"), case=k,
                        n=np.array([specs[i][0] for i in rows]), seed=np.array([specs[i][1] for i in rows]),
                        mu=np.array([specs[i][2] for i in rows]), ref_stop=np.array(stop), jitter=np.array(0.1),
                        residual=np.array(1e-6))
    print("batch cavities up to n =", max_n, ":", len(rows), "cases")


def write_channel_coarse(d):
    """The coarse k-epsilon channel (meshgen writes the same bytes every time)."""
    from sysu_cfd_parallel_gb300 import meshgen
    return os.path.dirname(meshgen.write_case(d, "channel", nx=50, ny=5, nz=5, jitter=0.15, seed=2026,
                                              steps=CHANNEL_COARSE_STEPS))


CHANNEL_COARSE_STEPS = 10
CHANNEL_COARSE_TR_STEPS = 3
CAVITY16G_STEPS = 3


def write_cavity16g_dual(d):
    """The perfect-gas cavity with the Dual scheme (meshgen writes the same bytes every time)."""
    from sysu_cfd_parallel_gb300 import meshgen
    return os.path.dirname(meshgen.write_case(d, "cavity", n=16, jitter=0.1, seed=9, density=1, wall_t=300,
                                              lid_t=330, time=(0.05, 1.0, 8, "Dual")))


def write_channel_coarse_tr(d):
    """The coarse channel, transient with the energy equation (meshgen writes the same bytes)."""
    from sysu_cfd_parallel_gb300 import meshgen
    return os.path.dirname(meshgen.write_case(d, "channel", nx=50, ny=5, nz=5, jitter=0.15, seed=2026,
                                              time=(0.1, 1.0, 6, "Euler"), energy=True, wall_t=290))


def channel_coarse_fixture():
    tmp = tempfile.mkdtemp()
    try:
        o = run_reference(write_channel_coarse(tmp), CHANNEL_COARSE_STEPS, [])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    keep = {"residual": o["residual"].reshape(-1, 10), "ksp": o["ksp"].reshape(-1, 4), "info": o["info"],
            "steps": np.array(CHANNEL_COARSE_STEPS)}
    for nm in ("U", "V", "W", "P", "TE", "ED"):
        keep[nm + "_norm"] = np.array(np.linalg.norm(o[nm]))
        keep[nm + "_sum"] = np.array(np.sum(o[nm]))
    os.makedirs(os.path.join(HERE, "channel_coarse"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "channel_coarse", "ref_ilu.npz"), **keep)
    print("channel_coarse iterations", o["residual"].size // 10, "solves", o["ksp"].size // 4)


def channel_coarse_tr_fixture():
    tmp = tempfile.mkdtemp()
    try:
        o = run_reference(write_channel_coarse_tr(tmp), CHANNEL_COARSE_TR_STEPS, [])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    keep = {"residual": o["residual"].reshape(-1, 10), "ksp": o["ksp"].reshape(-1, 4), "info": o["info"],
            "steps": np.array(CHANNEL_COARSE_TR_STEPS)}
    for nm in ("U", "V", "W", "P", "TE", "ED", "T", "R"):
        keep[nm + "_norm"] = np.array(np.linalg.norm(o[nm]))
        keep[nm + "_sum"] = np.array(np.sum(o[nm]))
    os.makedirs(os.path.join(HERE, "channel_coarse_tr"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "channel_coarse_tr", "ref_ilu.npz"), **keep)
    print("channel_coarse_tr outer iterations", o["residual"].size // 10, "solves", o["ksp"].size // 4)


def cavity16g_fixture():
    tmp = tempfile.mkdtemp()
    try:
        o = run_reference(write_cavity16g_dual(tmp), CAVITY16G_STEPS, [])
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    keep = {"residual": o["residual"].reshape(-1, 10), "ksp": o["ksp"].reshape(-1, 4), "info": o["info"],
            "steps": np.array(CAVITY16G_STEPS)}
    for nm in ("U", "V", "W", "P", "T", "R"):
        keep[nm + "_norm"] = np.array(np.linalg.norm(o[nm]))
        keep[nm + "_sum"] = np.array(np.sum(o[nm]))
    os.makedirs(os.path.join(HERE, "cavity16g_dual"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "cavity16g_dual", "ref_ilu.npz"), **keep)
    print("cavity16g_dual outer iterations", o["residual"].size // 10, "solves", o["ksp"].size // 4)


def main():
    build()
    cavity48_fixture()
    channel_coarse_fixture()
    channel_coarse_tr_fixture()
    cavity16g_fixture()
    tmp = tempfile.mkdtemp()
    os.makedirs(os.path.join(HERE, "cavity20"), exist_ok=True)
    for name, (steps, opts) in RUNS.items():
        d = write_cavity20(tmp) if name == "cavity20" else os.path.join(HERE, name)
        out_dir = os.path.join(HERE, name)
        for pc in ("ilu", "jacobi"):
            options = list(opts) + (["-pc_type", "jacobi"] if pc == "jacobi" else [])
            o = run_reference(d, steps, options)
            # the long run keeps its residual history, Krylov log and velocity / pressure only
            np.savez_compressed(os.path.join(out_dir, "ref_%s.npz" % pc),
                                **pack(o, steps, options, name != "cavity20"))
            print(name, pc, "iterations", o["residual"].size // 10, "solves", o["ksp"].size // 4)
    shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
