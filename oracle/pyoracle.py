"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU arm as the
checker; the product never imports it.  Parity is unpinned at the PETSc
boundary (see oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_cycas.so")

PC_NONE, PC_JACOBI, PC_ILU0, PC_POLY1, PC_POLY2, PC_POLY3, PC_POLY4, PC_POLY5 = 0, 1, 2, 3, 4, 5, 6, 7
KSP_GMRES, KSP_CG = 0, 1
VELOCITY, PRESSURE, SCALAR = 0, 1, 2

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_load.restype = C.c_void_p
        L.orc_load.argtypes = [C.c_char_p]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_last_error.restype = C.c_char_p
        L.orc_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
        L.orc_get_params.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        for f in (L.orc_get, L.orc_set):
            f.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_long]
        L.orc_geti.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p, C.c_long]
        L.orc_set_ksp.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.orc_set_ksp_type.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_set_ksp_perm.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_long]
        L.orc_set_libm_pow.argtypes = [C.c_void_p, C.c_int]
        L.orc_stage.argtypes = [C.c_void_p, C.c_char_p]
        L.orc_iterate.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_physics.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_time_step.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_csr_solve.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                    C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleCase:
    """One loaded case (param.in + gmsh mesh) in the CPU restatement."""

    def __init__(self, param_path: str):
        L = lib()
        h = L.orc_load(param_path.encode())
        if not h:
            raise RuntimeError("oracle load failed: " + L.orc_last_error().decode())
        self.h = C.c_void_p(h)
        d = (C.c_int * 8)()
        L.orc_dims(self.h, d)
        self.ncel, self.nfac, self.nbnd, self.nvrt, self.turb, self.nnz, self.max_step, self.cell_pref = list(d)

    def close(self):
        if self.h:
            lib().orc_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    _SIZES = None

    def _size(self, name):
        n, f, b = self.ncel, self.nfac, self.nbnd
        table = {
            "face_x": 3 * f, "face_n": 3 * f, "face_xpac": 3 * f, "face_xnac": 3 * f,
            "face_area": f, "face_lambda": f, "face_rlencos": f, "RUFace": f,
            "cell_vol": n, "cell_x": 3 * n, "bnd_distance": b, "bnd_shear": 3 * b,
            "dUdX": 3 * n, "dVdX": 3 * n, "dWdX": 3 * n, "dPdX": 3 * n, "dPhidX": 3 * n,
            "BRo": b, "BU": b, "BV": b, "BW": b, "BPre": b, "BTE": b, "BED": b,
            "Au_val": self.nnz, "Ap_val": self.nnz, "As_val": self.nnz, "residual": 10,
            "vert": 3 * self.nvrt, "BTem": b,
            "face_cell1": f, "face_cell2": f, "face_bnd": f, "face_vertices": 4 * f,
            "cell_nface": n, "cell_rid": n, "cell_face": 6 * n, "cell_cell": 6 * n, "cell_vertices": 8 * n,
            "bnd_face": b, "bnd_rid": b, "bnd_type": b, "bnd_vertices": 4 * b,
            "A_rowptr": n + 1, "A_col": self.nnz,
        }
        return table.get(name, n)

    def get(self, name):
        out = np.empty(self._size(name), dtype=np.float64)
        rc = lib().orc_get(self.h, name.encode(), _ptr(out), out.size)
        if rc != 0:
            raise KeyError(f"{name}: rc={rc} {lib().orc_last_error().decode()}")
        return out

    def geti(self, name):
        out = np.empty(self._size(name), dtype=np.int32)
        rc = lib().orc_geti(self.h, name.encode(), _ptr(out), out.size)
        if rc != 0:
            raise KeyError(f"{name}: rc={rc} {lib().orc_last_error().decode()}")
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        rc = lib().orc_set(self.h, name.encode(), _ptr(a), a.size)
        if rc != 0:
            raise KeyError(f"{name}: rc={rc} {lib().orc_last_error().decode()}")

    def params(self):
        urf = np.empty(8); g = np.empty(3)
        lib().orc_get_params(self.h, _ptr(urf), _ptr(g))
        return urf, g

    def set_ksp(self, which, pc=PC_ILU0, restart=30, rtol=-1.0, maxit=-1, perm=None, ksp_type=None):
        lib().orc_set_ksp(self.h, which, pc, restart, rtol, maxit)
        if ksp_type is not None:
            lib().orc_set_ksp_type(self.h, which, ksp_type)
        if perm is not None:
            p = np.ascontiguousarray(perm, dtype=np.int32)
            lib().orc_set_ksp_perm(self.h, which, _ptr(p), p.size)

    def set_libm_pow(self, flag=True):
        """TE^1.5 of the wall function through the C library's pow, as the reference's own build
        computes it, instead of the once-rounded value the GPU computes."""
        lib().orc_set_libm_pow(self.h, 1 if flag else 0)

    def stage(self, name):
        rc = lib().orc_stage(self.h, name.encode())
        if rc != 0:
            raise RuntimeError(f"stage {name}: {lib().orc_last_error().decode()}")

    def physics(self):
        """dict of the transient / energy / density switches read from param.in."""
        iv = (C.c_int * 6)()
        dv = (C.c_double * 4)()
        lib().orc_physics(self.h, iv, dv)
        return {"steady": bool(iv[0]), "time_scheme": iv[1], "max_outer": iv[2], "energy": bool(iv[3]),
                "density": iv[4], "max_step": iv[5], "dt": dv[0], "total_time": dv[1], "cur_time": dv[2],
                "pressure_reference": dv[3]}

    def time_step(self, cap=64):
        """One physical time step; returns dict(n, resmax [n], residual [n,10], ksp_its [n,8],
        ksp_reason [n,8])."""
        rm = np.zeros(cap); res = np.zeros((cap, 10))
        its = np.zeros((cap, 8), dtype=np.int32); rs = np.zeros((cap, 8), dtype=np.int32)
        n = lib().orc_time_step(self.h, cap, _ptr(rm), _ptr(res), _ptr(its), _ptr(rs))
        if n < 0:
            raise RuntimeError("oracle time step failed: " + lib().orc_last_error().decode())
        k = min(n, cap)
        return {"n": n, "resmax": rm[:k], "residual": res[:k], "ksp_its": its[:k], "ksp_reason": rs[:k]}

    def iterate(self, nsteps):
        res = np.zeros((nsteps, 10)); rm = np.zeros(nsteps)
        its = np.zeros((nsteps, 8), dtype=np.int32); rs = np.zeros((nsteps, 8), dtype=np.int32)
        rc = lib().orc_iterate(self.h, nsteps, _ptr(res), _ptr(rm), _ptr(its), _ptr(rs))
        if rc != nsteps:
            raise RuntimeError(f"oracle iteration {-rc} failed: {lib().orc_last_error().decode()}")
        return {"residual": res, "resmax": rm, "ksp_its": its, "ksp_reason": rs}


def csr_solve(rowptr, col, val, b, x0=None, pc=PC_JACOBI, restart=30, rtol=1e-8, maxit=1000, guess_zero=True,
              ksp_type=KSP_GMRES):
    n = len(rowptr) - 1
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    vl = np.ascontiguousarray(val, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    its = C.c_int(); reason = C.c_int(); rn = C.c_double()
    rc = lib().orc_csr_solve(n, _ptr(rp), _ptr(cl), _ptr(vl), _ptr(bb), _ptr(x), ksp_type, pc, restart, rtol, maxit,
                             1 if guess_zero else 0, C.byref(its), C.byref(reason), C.byref(rn))
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())
    return x, its.value, reason.value, rn.value


# ---------------------------------------------------------------- result files (restatement)
# Pure-Python renderings of the reference's writers, used by the tests as the checker of the
# library's files.  Python's own float formatting (not the C library's printf) renders each
# number, so agreement is a check of both.

def _c_float_text(fmt, x):
    """printf conversion of one double as glibc prints it (a NaN with the sign bit set is "-nan")."""
    x = float(x)
    if x != x:
        neg = np.signbit(x)
        w = fmt[1:].split(".")[0].rstrip("fg")
        s = ("-nan" if neg else "nan")
        return s.rjust(int(w)) if w else s
    return fmt % x


def _block(vals):
    """OutArray2File (NS/navierIO.cpp:2-17): "%19.5f " on a 20-character stride, "\\n" after
    every fifth value and after the block."""
    out = []
    n = len(vals)
    for i, v in enumerate(vals):
        s = _c_float_text("%19.5f", v) + " "
        fifth = i % 5 == 4
        if len(s) > 20 and (i != n - 1 or fifth):
            s = s[:20]
        out.append(s)
        if fifth:
            out.append("\n")
    out.append("\n")
    return "".join(out)


def tecplot_text(vert, cell_vertices, f, turb, density=0, pref=1.01325e5):
    """Output2Tecplot (NS/navierIO.cpp:161-283) at one rank: ``vert`` [nvrt, 3] or flat,
    ``cell_vertices`` zero-based [ncel * 8], ``f`` a dict of cell fields P U V W R T VisLam VisTur
    [TE ED]; with ``density`` 1 the Ma column is the Mach number (gamma 1.4)."""
    vert = np.asarray(vert, dtype=np.float64).reshape(-1, 3)
    cv = np.asarray(cell_vertices).reshape(-1, 8)
    n = cv.shape[0]
    nvar = 8 if turb == 1 else 6
    head = 'variables= "x", "y", "z", "p", "u", "v", "w", "ro", "T","Ma","mu" '
    if turb == 1:
        head += '"te", "ed"'
    parts = [head + "\n",
             "ZONE N=%d, E=%d, VARLOCATION=([1-3]=NODAL,[4-%d]=CELLCENTERED) DATAPACKING=BLOCK, ZONETYPE=FEBRICK\n"
             % (vert.shape[0], n, 3 + nvar + 2)]
    for d in range(3):
        parts.append(_block(vert[:, d]))
    for nm in ("P", "U", "V", "W", "R", "T"):
        parts.append(_block(f[nm]))
    U, V, W = (np.asarray(f[k], dtype=np.float64) for k in ("U", "V", "W"))
    if density == 1:
        P, R = (np.asarray(f[k], dtype=np.float64) for k in ("P", "R"))
        parts.append(_block(np.sqrt((U * U + V * V + W * W) / (1.4 * (P + pref) / R))))
    else:
        parts.append(_block(np.sqrt(U * U + V * V + W * W)))
    parts.append(_block(np.asarray(f["VisLam"]) + np.asarray(f["VisTur"])))
    if turb == 1:
        parts.append(_block(f["TE"]))
        parts.append(_block(f["ED"]))
    parts.append("".join("%d %d %d %d %d %d %d %d\n " % tuple(int(v) + 1 for v in row) for row in cv))
    return "".join(parts)


def grid_text(vert, cell_vertices):
    """OutputGrid (NS/navierIO.cpp:58-128) at one rank: no interface vertices."""
    vert = np.asarray(vert, dtype=np.float64).reshape(-1, 3)
    cv = np.asarray(cell_vertices).reshape(-1, 8)
    parts = ['title = "cycas partition grid"\nvariables="x","y","z","p"\n',
             "zone n=%d, e=%d, f=fepoint, et=BRICK\n" % (vert.shape[0], cv.shape[0])]
    parts += ["%f %f %f %f\n" % (x, y, z, 0.0) for x, y, z in vert]
    parts += ["%8d %8d %8d %8d %8d %8d %8d %8d\n" % tuple(int(v) + 1 for v in row) for row in cv]
    return "".join(parts)


def geo_bytes(vert, cell_vertices):
    """OutputGridBinary (NS/navierIO.cpp:29-55) at rank 0 of one partition."""
    vert = np.asarray(vert, dtype="<f8").reshape(-1, 3)
    cv = np.asarray(cell_vertices, dtype="<i4").reshape(-1, 8)
    return (np.array([0, 1, cv.shape[0], vert.shape[0]], dtype="<i4").tobytes() + vert.tobytes()
            + (cv + 1).astype("<i4").tobytes())


def data_bytes(f, turb):
    """Output2TecplotBinary (NS/navierIO.cpp:132-159)."""
    names = ["P", "U", "V", "W", "R", "T"] + (["TE", "ED"] if turb == 1 else [])
    return (np.array([0, len(names)], dtype="<i4").tobytes()
            + b"".join(np.asarray(f[k], dtype="<f8").tobytes() for k in names))


def backup_text(f, turb):
    """WriteBackupFile (NS/navierIO.cpp:370-387): ostream's default conversion is %g."""
    g = lambda x: _c_float_text("%g", x)
    n = len(f["U"])
    out = []
    for i in range(n):
        out.append(" ".join(g(f[k][i]) for k in ("R", "U", "V", "W", "P", "T", "R", "VisLam")) + "\n")
        if turb == 1:
            out.append(" ".join(g(f[k][i]) for k in ("VisTur", "TE", "ED")) + "\n")
    return "".join(out)
