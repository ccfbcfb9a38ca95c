"""Host-side mirror of the reference's solver seams over the C ABI.

``NavierStokesSolver`` follows NS/navier.h:30-226: a case is read from a ``param.in`` with
its gmsh mesh, ``CalculateVelocity`` / ``CalculatePressure`` / ``UpdateTurKEpsilon`` run
the corresponding stages on the GPU and ``NSSolve`` runs the steady outer loop
(NS/navier.cpp:17-156).  A Krylov failure raises ``ConvergeError`` as the reference does
(BasicType.h:62-68).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


class ConvergeError(RuntimeError):
    """Raised when a Krylov solve ends with a negative converged reason."""

    def __init__(self, iter_: int, residual: float, varname: str):
        super().__init__(f"{varname} not converge in iter: {iter_}, res {residual:f}")
        self.iter = iter_
        self.residual = residual
        self.varname = varname


_SOLVE_NAMES = ("Un", "Vn", "Wn", "Pn", "Tn", "ED", "?", "?")


class Case:
    """param.in + mesh loaded by the library's host code (no GPU needed); ``msh_binary`` reads
    the gridfile as the compressed binary gmsh form (the reference's -mshBinary switch)."""

    def __init__(self, param_path: str, msh_binary: bool = False):
        L = capi.load()
        h = C.c_void_p()
        flags = capi.LOAD_MSH_BINARY if msh_binary else 0
        capi.check(L.cycas_case_load_ex(param_path.encode(), flags, C.byref(h)))
        self._h = h
        d = (C.c_int64 * 8)()
        capi.check(L.cycas_case_dims(h, d))
        (self.ncel, self.nfac, self.nbnd, self.nvrt, self.turb_model, self.max_step, self.cell_pressure_ref,
         self.nnz) = [int(x) for x in d]
        rs = C.c_double()
        urf = (C.c_double * 8)()
        g = (C.c_double * 3)()
        capi.check(L.cycas_case_params(h, C.byref(rs), urf, g))
        self.residual_steady = rs.value
        self.urf = list(urf)
        self.gravity = list(g)
        iv, dv = (C.c_int32 * 6)(), (C.c_double * 3)()
        capi.check(L.cycas_case_physics(h, iv, dv))
        self.steady, self.time_scheme, self.max_outer = bool(iv[0]), int(iv[1]), int(iv[2])
        self.solve_energy, self.density_model = bool(iv[3]), int(iv[4])
        self.dt, self.total_time, self.pressure_reference = float(dv[0]), float(dv[1]), float(dv[2])
        no, rst = C.c_int32(), C.c_int32()
        capi.check(L.cycas_case_output(h, C.byref(no), C.byref(rst)))
        self.noutput = no.value
        self.restart = bool(rst.value)
        self.param_path = param_path

    def get_field(self, name: str) -> np.ndarray:
        """Host arrays of the loaded case: ``vert`` [3*nvrt] or an initial cell field."""
        out = np.empty(3 * self.nvrt if name == "vert" else self.ncel, dtype=np.float64)
        capi.check(capi.load().cycas_case_get_field(self._h, name.encode(), capi.ptr(out), out.size))
        return out

    def OutputGrid(self, path: str = "tec/grid.dat") -> None:
        """ASCII Tecplot grid (NS/navierIO.cpp:58-128)."""
        capi.check(capi.load().cycas_write_grid(self._h, path.encode(), 0))

    def OutputGridBinary(self, path: str = "tec/geo") -> None:
        """Binary geometry (NS/navierIO.cpp:29-55)."""
        capi.check(capi.load().cycas_write_grid(self._h, path.encode(), 1))

    def get_int(self, name: str) -> np.ndarray:
        sizes = {"face_cell1": self.nfac, "face_cell2": self.nfac, "face_bnd": self.nfac,
                 "face_vertices": 4 * self.nfac, "cell_nface": self.ncel, "cell_face": 6 * self.ncel,
                 "cell_cell": 6 * self.ncel, "cell_vertices": 8 * self.ncel, "cell_rid": self.ncel,
                 "bnd_face": self.nbnd, "bnd_rid": self.nbnd, "bnd_type": self.nbnd, "bnd_vertices": 4 * self.nbnd}
        out = np.empty(sizes[name], dtype=np.int32)
        capi.check(capi.load().cycas_case_get_int(self._h, name.encode(), capi.ptr(out), out.size))
        return out

    def footprint(self) -> float:
        """Estimated device bytes of this case in a batch (cycas_footprint_estimate)."""
        return capi.load().cycas_footprint_estimate(self._h)

    def close(self):
        if self._h:
            capi.load().cycas_case_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NavierStokesSolver:
    """One device-resident case.  ``options`` is a ``capi.Options``."""

    def __init__(self, case: Case, options: capi.Options | None = None):
        L = capi.load()
        self.case = case
        self.options = options or capi.default_options()
        h = C.c_void_p()
        capi.check(L.cycas_create_from_case(case._h, C.byref(self.options), C.byref(h)))
        self._h = h
        self.step = 0
        self.cur_time = 0.0
        self.Residual = np.zeros(10)
        self.last_stats = None

    # ---- arrays
    def _size(self, name):
        n, f, b = self.case.ncel, self.case.nfac, self.case.nbnd
        three = {"dUdX", "dVdX", "dWdX", "dPdX", "dPhidX", "cell_x"}
        faces = {"RUFace", "face_area", "face_lambda", "face_rlencos"}
        faces3 = {"face_x", "face_n", "face_xpac", "face_xnac"}
        bnd = {"BRo", "BU", "BV", "BW", "BPre", "BTE", "BED", "BTem", "bnd_distance"}
        if name in three:
            return 3 * n
        if name in faces:
            return f
        if name in faces3:
            return 3 * f
        if name in bnd:
            return b
        if name == "bnd_shear":
            return 3 * b
        if name == "old_uvw":
            return 3 * n
        if name in ("Au_val", "Ap_val", "As_val"):
            return self.case.nnz
        return n

    def get(self, name: str) -> np.ndarray:
        out = np.empty(self._size(name), dtype=np.float64)
        capi.check(capi.load().cycas_get_field(self._h, name.encode(), capi.ptr(out), out.size))
        return out

    def set(self, name: str, values) -> None:
        a = np.ascontiguousarray(values, dtype=np.float64)
        capi.check(capi.load().cycas_set_field(self._h, name.encode(), capi.ptr(a), a.size))

    @staticmethod
    def _pack(arrays: dict, host_to_device: bool):
        names = list(arrays)
        k = len(names)
        nm = (C.c_char_p * k)(*[x.encode() for x in names])
        ptrs = (C.c_void_p * k)()
        sizes = (C.c_int64 * k)()
        for q, x in enumerate(names):
            a = arrays[x]
            if a.dtype != np.float64 or not a.flags.c_contiguous or (not host_to_device and not a.flags.writeable):
                raise TypeError(f"{x}: contiguous float64 array required")
            ptrs[q] = a.ctypes.data
            sizes[q] = a.size
        return k, nm, ptrs, sizes

    def _many(self, fn, arrays: dict, host_to_device: bool):
        capi.check(fn(self._h, *self._pack(arrays, host_to_device)))

    def set_fields(self, arrays: dict) -> None:
        """Uploads several named arrays with one synchronisation (cycas_set_fields)."""
        self._many(capi.load().cycas_set_fields, arrays, True)

    def get_fields(self, arrays: dict) -> None:
        """Fills the given arrays from the named device arrays with one synchronisation."""
        self._many(capi.load().cycas_get_fields, arrays, False)

    def get_int(self, name: str) -> np.ndarray:
        n = self.case.ncel + 1 if name == "A_rowptr" else self.case.nnz
        out = np.empty(n, dtype=np.int32)
        capi.check(capi.load().cycas_get_int(self._h, name.encode(), capi.ptr(out), out.size))
        return out

    # ---- reference-facing operations
    def _raise_for(self, rc, stats):
        if rc == capi.CYCAS_NOT_CONVERGED and stats is not None and stats.failed_solve >= 0:
            k = stats.failed_solve
            raise ConvergeError(stats.its[k], stats.rnorm[k], _SOLVE_NAMES[k])
        capi.check(rc)

    def stage(self, name: str) -> None:
        capi.check(capi.load().cycas_run_stage(self._h, name.encode()))

    def CalculateVelocity(self):
        self.stage("calculate_velocity")

    def CalculatePressure(self):
        self.stage("calculate_pressure")

    def UpdateTurKEpsilon(self):
        self.stage("keps")

    def simple_iteration(self):
        res = (C.c_double * 10)()
        rm = C.c_double()
        st = capi.IterStats()
        rc = capi.load().cycas_simple_iteration(self._h, res, C.byref(rm), C.byref(st))
        self.last_stats = st
        self._raise_for(rc, st)
        self.step += 1
        self.Residual = np.array(list(res))
        return rm.value

    def simple_iteration_io(self, inputs: dict, outputs: dict):
        """One iteration whose state comes from and goes to host arrays (cycas_simple_iteration_io):
        the uploads of `inputs` and downloads into `outputs` overlap the iteration where its
        stages allow; the same results as set_fields + simple_iteration + get_fields."""
        res = (C.c_double * 10)()
        rm = C.c_double()
        st = capi.IterStats()
        ni, inm, ip, isz = self._pack(inputs, True)
        no, onm, op, osz = self._pack(outputs, False)
        rc = capi.load().cycas_simple_iteration_io(self._h, ni, inm, ip, isz, no, onm, op, osz, res, C.byref(rm),
                                                   C.byref(st))
        self.last_stats = st
        self._raise_for(rc, st)
        self.step += 1
        self.Residual = np.array(list(res))
        return rm.value

    def iterate(self, n: int):
        """n iterations; returns dict(residual [n,10], resmax [n], ksp_its [n,8], ksp_reason [n,8])."""
        res = np.zeros((n, 10)); rm = np.zeros(n)
        its = np.zeros((n, 8), dtype=np.int32); rs = np.zeros((n, 8), dtype=np.int32)
        rc = capi.load().cycas_simple_iterations(self._h, n, capi.ptr(res), capi.ptr(rm), capi.ptr(its), capi.ptr(rs))
        capi.check(rc)
        self.step += n
        return {"residual": res, "resmax": rm, "ksp_its": its, "ksp_reason": rs}

    def solve_steady(self, max_step: int | None = None, residual_steady: float | None = None):
        """The steady loop of NSSolve without its result files (cycas_solve_steady): iterations
        until ResMax < residual_steady or max_step of them; returns dict(iterations, residual
        [n,10], resmax [n], ksp_its [n,8], ksp_reason [n,8]).  A failed solve raises as
        ``iterate`` does, after the iterations that ran are counted."""
        max_step = self.case.max_step if max_step is None else max_step
        tol = self.case.residual_steady if residual_steady is None else residual_steady
        res = np.zeros((max_step, 10)); rm = np.zeros(max_step)
        its = np.zeros((max_step, 8), dtype=np.int32); rs = np.zeros((max_step, 8), dtype=np.int32)
        n = C.c_int32(0)
        rc = capi.load().cycas_solve_steady(self._h, max_step, tol, max_step, C.byref(n), capi.ptr(res),
                                            capi.ptr(rm), capi.ptr(its), capi.ptr(rs))
        k = n.value
        self.step += k
        capi.check(rc)
        return {"iterations": k, "residual": res[:k], "resmax": rm[:k], "ksp_its": its[:k], "ksp_reason": rs[:k]}

    def save_restart_point(self) -> None:
        """Keeps a device copy of the whole state (cycas_restart_point SAVE)."""
        capi.check(capi.load().cycas_restart_point(self._h, 0))

    def restore_restart_point(self) -> None:
        """Returns to the state of the last save_restart_point (device-to-device copies)."""
        capi.check(capi.load().cycas_restart_point(self._h, 1))

    # ---- DataPartition::solve* (MPIStructure.h:224-228) on the last assembled systems; the
    # arrays are solved in place, as the reference writes into the caller's arrays
    def _solved(self, rc, st, name):
        self.last_stats = st
        if rc == capi.CYCAS_NOT_CONVERGED and st.failed_solve >= 0:
            k = st.failed_solve
            raise ConvergeError(st.its[k], st.rnorm[k], name)
        capi.check(rc)
        return st

    def solveVelocity_GMRES(self, tol: float, maxIter: int, xu: np.ndarray, xv: np.ndarray, xw: np.ndarray):
        st = capi.IterStats()
        for x in (xu, xv, xw):
            if x.dtype != np.float64 or not x.flags.c_contiguous:
                raise TypeError("solution arrays must be contiguous float64")
        rc = capi.load().cycas_solve_velocity(self._h, tol, maxIter, capi.ptr(xu), capi.ptr(xv), capi.ptr(xw),
                                              C.byref(st))
        return self._solved(rc, st, "Un")

    def solvePressureCorrection(self, tol: float, maxIter: int, xp: np.ndarray, isSymmetric: bool = True):
        st = capi.IterStats()
        if xp.dtype != np.float64 or not xp.flags.c_contiguous:
            raise TypeError("solution array must be contiguous float64")
        rc = capi.load().cycas_solve_pressure(self._h, tol, maxIter, capi.ptr(xp), 1 if isSymmetric else 0,
                                              C.byref(st))
        return self._solved(rc, st, "Pn")

    def solveScarlar_GMRES(self, tol: float, maxIter: int, xs: np.ndarray):
        st = capi.IterStats()
        if xs.dtype != np.float64 or not xs.flags.c_contiguous:
            raise TypeError("solution array must be contiguous float64")
        rc = capi.load().cycas_solve_scalar(self._h, tol, maxIter, capi.ptr(xs), C.byref(st))
        return self._solved(rc, st, "scalar")

    def time_step(self, cap: int = 64):
        """One physical time step of a transient case (cycas_time_step): returns dict(n,
        resmax [n], residual [n, 10], ksp_its [n, 8], ksp_reason [n, 8], cur_time)."""
        n = C.c_int32()
        t = C.c_double()
        rm = np.zeros(cap); res = np.zeros((cap, 10))
        its = np.zeros((cap, 8), dtype=np.int32); rs = np.zeros((cap, 8), dtype=np.int32)
        rc = capi.load().cycas_time_step(self._h, cap, C.byref(n), capi.ptr(res), capi.ptr(rm), capi.ptr(its),
                                         capi.ptr(rs), C.byref(t))
        k = min(n.value, cap)
        self.step += 1
        self.cur_time = t.value
        if rc == capi.CYCAS_NOT_CONVERGED and k > 0:
            row = its[k - 1]
            bad = [q for q in range(8) if rs[k - 1][q] < 0]
            q = bad[0] if bad else 0
            raise ConvergeError(int(row[q]), 0.0, _SOLVE_NAMES[q])
        capi.check(rc)
        return {"n": n.value, "resmax": rm[:k], "residual": res[:k], "ksp_its": its[:k], "ksp_reason": rs[:k],
                "cur_time": t.value}

    # ---- result files (NS/navierIO.cpp); k is the case of a batch, 0 otherwise
    def _case_handle(self, k: int):
        if k != 0:
            raise IndexError("a single-case solver has case 0 only")
        return self.case._h

    def Output2Tecplot(self, path: str = "tec/res0000.dat", k: int = 0) -> None:
        """ASCII Tecplot result of the current fields (NS/navierIO.cpp:161-283)."""
        capi.check(capi.load().cycas_write_tecplot(self._h, k, self._case_handle(k), path.encode()))

    def Output2TecplotBinary(self, path: str = "tec/data", k: int = 0) -> None:
        """Binary cell fields P U V W R T [TE ED] (NS/navierIO.cpp:132-159)."""
        capi.check(capi.load().cycas_write_data(self._h, k, path.encode()))

    def WriteBackupFile(self, path: str = "localGeometryBackup_0/res.sav", k: int = 0) -> None:
        """Restart file (NS/navierIO.cpp:370-387)."""
        capi.check(capi.load().cycas_write_backup(self._h, k, path.encode()))

    def ReadBackupFile(self, path: str = "res.sav", k: int = 0) -> None:
        """Sets the cell fields from a restart file (NS/navierIO.cpp:389-404)."""
        capi.check(capi.load().cycas_read_backup(self._h, k, path.encode()))

    def dump_begin(self, tecplot: str | None = None, data: str | None = None, backup: str | None = None,
                   k: int = 0) -> None:
        """Starts an asynchronous dump of the current fields to the given files (cycas_dump_begin):
        the solve may continue at once; ``dump_wait`` collects the status."""
        kinds = ((capi.DUMP_TECPLOT if tecplot else 0) | (capi.DUMP_DATA if data else 0)
                 | (capi.DUMP_BACKUP if backup else 0))
        enc = lambda x: x.encode() if x else None
        capi.check(capi.load().cycas_dump_begin(self._h, k, self._case_handle(k) if tecplot else None, kinds,
                                                enc(tecplot), enc(data), enc(backup)))

    def dump_wait(self) -> None:
        capi.check(capi.load().cycas_dump_wait(self._h))

    def NSSolve(self, max_step: int | None = None, residual_steady: float | None = None, callback=None,
                output_dir: str | None = None, out_binary: bool = False, noutput: int | None = None,
                async_output: bool = True):
        """Outer loop (NS/navier.cpp:52-141).  Steady: SIMPLE iterations until ResMax <
        ResidualSteady.  Transient: time steps (each ``time_step``) until the clock reaches
        total_time.

        With ``output_dir`` the reference's files are written under it at the reference's
        cadence: the grid before the loop (tec/geo with ``out_binary``, else tec/grid.dat;
        geometry.cpp:209-213); after step s (1-based) with (s - 1) % noutput == 0 the backup
        localGeometryBackup_0/res.sav and tec/data (``out_binary``) or tec/res0000.dat
        (navier.cpp:113-122, 161-199); after the loop tec/res0000.dat (navier.cpp:149).  With
        ``async_output`` the in-loop files are written by asynchronous dumps of the step's fields
        (same bytes) while the next iterations run.
        """
        import os

        max_step = self.case.max_step if max_step is None else max_step
        tol = self.case.residual_steady if residual_steady is None else residual_steady
        nout = max(1, (self.case.noutput if noutput is None else noutput))
        if output_dir is not None:
            tec = os.path.join(output_dir, "tec")
            bak = os.path.join(output_dir, "localGeometryBackup_0")
            os.makedirs(tec, exist_ok=True)
            os.makedirs(bak, exist_ok=True)
            if out_binary:
                self.case.OutputGridBinary(os.path.join(tec, "geo"))
            else:
                self.case.OutputGrid(os.path.join(tec, "grid.dat"))
        rm = None
        transient = not getattr(self.case, "steady", True)
        for step in range(1, max_step + 1):
            if transient:  # one physical time step of outer iterations (navier.cpp:52-111)
                r = self.time_step()
                rm = float(r["resmax"][-1]) if r["n"] else 0.0
                self.Residual = r["residual"][-1] if r["n"] else np.zeros(10)
            else:
                rm = self.simple_iteration()
            if callback:
                callback(self.step, rm, self.Residual)
            if output_dir is not None and (step - 1) % nout == 0:
                backup = os.path.join(bak, "res.sav")
                data = os.path.join(tec, "data") if out_binary else None
                res = None if out_binary else os.path.join(tec, "res0000.dat")
                if async_output:
                    self.dump_begin(tecplot=res, data=data, backup=backup)
                else:
                    self.WriteBackupFile(backup)
                    if out_binary:
                        self.Output2TecplotBinary(data)
                    else:
                        self.Output2Tecplot(res)
            if transient:
                if self.cur_time >= self.case.total_time:
                    break
            elif rm < tol:
                break
        if output_dir is not None:
            if async_output:
                self.dump_wait()
            self.Output2Tecplot(os.path.join(tec, "res0000.dat"))
        return rm

    # ---- measurement hooks
    def stream_handle(self) -> int:
        s = C.c_void_p()
        capi.check(capi.load().cycas_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def set_profiling(self, on: bool) -> None:
        capi.check(capi.load().cycas_set_profiling(self._h, 1 if on else 0))

    def set_graph(self, on: bool) -> None:
        """Replay each iteration as one captured CUDA graph (exclusive with profiling)."""
        capi.check(capi.load().cycas_set_graph(self._h, 1 if on else 0))

    def amg_levels(self):
        """(rows, nnz) per level of the pressure AMG hierarchy, fine to coarse."""
        nl = C.c_int32()
        rows = np.zeros(16, dtype=np.int32)
        nnz = np.zeros(16, dtype=np.int32)
        capi.check(capi.load().cycas_get_amg_levels(self._h, 16, C.byref(nl), capi.ptr(rows), capi.ptr(nnz)))
        k = min(nl.value, 16)
        return rows[:k].copy(), nnz[:k].copy()

    def reset_profile(self) -> None:
        capi.check(capi.load().cycas_reset_profile(self._h))

    def profile(self) -> dict:
        p = capi.Profile()
        capi.check(capi.load().cycas_get_profile(self._h, C.byref(p)))
        return {"kernel_launches": p.kernel_launches, "krylov_launches": list(p.krylov_launches),
                "krylov_iters": list(p.krylov_iters), "krylov_ms": list(p.krylov_ms), "assembly_ms": p.assembly_ms}

    def close(self):
        if getattr(self, "_h", None):
            capi.load().cycas_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def csr_solve(rowptr, col, val, b, x0=None, pc=capi.PC_JACOBI, restart=30, rtol=1e-8, maxit=1000,
              guess_zero=True, ksp_type=capi.KSP_GMRES):
    """Standalone GPU GMRES on a host CSR system (cycas_csr_solve)."""
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    vl = np.ascontiguousarray(val, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    n = rp.size - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    k = capi.KspOptions(type=ksp_type, restart=restart, pc=pc, rtol=0.0, maxit=0)
    st = capi.SolveStats()
    rc = capi.load().cycas_csr_solve(n, capi.ptr(rp), capi.ptr(cl), capi.ptr(vl), capi.ptr(bb), capi.ptr(x),
                                     C.byref(k), rtol, maxit, 1 if guess_zero else 0, C.byref(st))
    if rc not in (capi.CYCAS_OK, capi.CYCAS_NOT_CONVERGED):
        capi.check(rc)
    return x, st.its, st.reason, st.rnorm


class _UnionSizes:
    """Sizes of the concatenated mesh of a batch (what NavierStokesSolver reads off a Case)."""

    def __init__(self, cases):
        self.ncel = sum(c.ncel for c in cases)
        self.nfac = sum(c.nfac for c in cases)
        self.nbnd = sum(c.nbnd for c in cases)
        self.nnz = sum(c.nnz for c in cases)
        self.turb_model = cases[0].turb_model
        self.max_step = max(c.max_step for c in cases)
        self.residual_steady = cases[0].residual_steady


def batch_options(pc=capi.PC_JACOBI, restart=30, device=0) -> capi.Options:
    """The reference's Krylov methods and tolerances, AMG for the pressure correction (required
    by batches)."""
    o = capi.default_options(pc=pc, restart=restart, device=device)
    o.ksp[capi.SYS_PRESSURE].pc = capi.PC_AMG
    return o


class Batch(NavierStokesSolver):
    """Independent cases advanced together on one device (cycas_batch_*).

    Fields are the cases' fields concatenated; ``case_field(name, c)`` slices one case.
    """

    def __init__(self, cases, options: capi.Options | None = None):
        L = capi.load()
        self.cases = list(cases)
        self.case = _UnionSizes(self.cases)
        self.options = options or batch_options()
        handles = (C.c_void_p * len(self.cases))(*[c._h.value for c in self.cases])
        h = C.c_void_p()
        capi.check(L.cycas_batch_create(handles, len(self.cases), C.byref(self.options), C.byref(h)))
        self._h = h
        n = C.c_int32()
        capi.check(L.cycas_batch_size(h, C.byref(n)))
        self.ncases = n.value
        self.cell0 = np.zeros(self.ncases + 1, dtype=np.int32)
        self.bnd0 = np.zeros(self.ncases + 1, dtype=np.int32)
        capi.check(L.cycas_batch_offsets(h, 0, capi.ptr(self.cell0)))
        capi.check(L.cycas_batch_offsets(h, 1, capi.ptr(self.bnd0)))
        self.step = 0
        self.last_stats = None

    def _case_handle(self, k: int):
        return self.cases[k]._h

    def autotune(self, iters: int = 1):
        """Times the team schedules (CTA count x row-share factor) over `iters` real iterations
        each and keeps the fastest; returns (grid, factor, ms per iteration)."""
        g, f, ms = C.c_int32(), C.c_double(), C.c_double()
        capi.check(capi.load().cycas_batch_autotune(self._h, iters, C.byref(g), C.byref(f), C.byref(ms)))
        self.step += 9 * iters
        return g.value, f.value, ms.value

    def case_field(self, name: str, c: int) -> np.ndarray:
        a = self.get(name)
        bnd = {"BRo", "BU", "BV", "BW", "BPre", "BTE", "BED", "BTem", "bnd_distance"}
        off = self.bnd0 if name in bnd else self.cell0
        return a[off[c]:off[c + 1]].copy()

    def iterate(self, n: int):
        """n iterations of every case; returns dict(resmax [n, ncases], ksp_its [n, ncases, 8],
        ksp_reason [n, ncases, 8], residual [n, ncases, 10])."""
        L = capi.load()
        nc = self.ncases
        rm = np.zeros((n, nc))
        its = np.zeros((n, nc, 8), dtype=np.int32)
        rs = np.zeros((n, nc, 8), dtype=np.int32)
        res = np.zeros((n, nc, 10))
        for k in range(n):
            rc = L.cycas_batch_iteration(self._h, capi.ptr(rm[k]), capi.ptr(its[k]), capi.ptr(rs[k]))
            capi.check(rc)
            capi.check(L.cycas_batch_residuals(self._h, capi.ptr(res[k])))
            self.step += 1
        return {"resmax": rm, "ksp_its": its, "ksp_reason": rs, "residual": res}


class Server:
    """Continuous-batching request server (cycas_server_*): submit param files, step, poll."""

    def __init__(self, hbm_budget_gb: float = 150.0, residual_tol: float = 1e-6, max_iters: int = 10000,
                 keep_fields: bool = False, options: capi.Options | None = None):
        L = capi.load()
        self.options = options or batch_options()
        h = C.c_void_p()
        capi.check(L.cycas_server_create(C.byref(self.options), hbm_budget_gb * 1e9, residual_tol, max_iters,
                                         1 if keep_fields else 0, C.byref(h)))
        self._h = h
        self.results = {}

    @staticmethod
    def clock() -> float:
        return capi.load().cycas_server_clock()

    def set_graph(self, on: bool) -> None:
        """Replay each batch's iterations as one CUDA graph (cycas_server_set_graph)."""
        capi.check(capi.load().cycas_server_set_graph(self._h, 1 if on else 0))

    def set_max_cells(self, max_cells: float) -> None:
        """Admit requests only while the active requests' cells stay within max_cells (0: no
        cap; cycas_server_set_max_cells)."""
        capi.check(capi.load().cycas_server_set_max_cells(self._h, float(max_cells)))

    def set_async_rebuild(self, on: bool) -> None:
        """Build new batches on a worker thread while the current ones keep iterating
        (cycas_server_set_async_rebuild)."""
        capi.check(capi.load().cycas_server_set_async_rebuild(self._h, 1 if on else 0))

    def submit(self, param_path: str) -> int:
        i = C.c_int64()
        rc = capi.load().cycas_server_submit(self._h, param_path.encode(), C.byref(i))
        if rc != capi.CYCAS_OK:
            raise capi.CycasError(rc, capi.load().cycas_server_last_error(self._h).decode())
        return i.value

    def step(self):
        """Admit, re-form batches, one iteration of every active case, retire; returns
        (active, queued) and records finished requests in ``results``."""
        L = capi.load()
        a, q = C.c_int32(), C.c_int32()
        rc = L.cycas_server_step(self._h, C.byref(a), C.byref(q))
        if rc != capi.CYCAS_OK:
            raise capi.CycasError(rc, L.cycas_server_last_error(self._h).decode())
        buf = (capi.RequestResult * 256)()
        while True:
            n = C.c_int32()
            capi.check(L.cycas_server_poll(self._h, buf, 256, C.byref(n)))
            for k in range(n.value):
                r = buf[k]
                self.results[r.id] = {"status": r.status, "iterations": r.iterations, "ncel": r.ncel,
                                      "t_arrival": r.t_arrival, "t_admit": r.t_admit, "t_done": r.t_done,
                                      "resmax": r.resmax}
            if n.value < 256:
                break
        return a.value, q.value

    def result_field(self, rid: int, name: str, n: int) -> np.ndarray:
        out = np.empty(n)
        capi.check(capi.load().cycas_server_result_field(self._h, rid, name.encode(), capi.ptr(out), n))
        return out

    def stats(self) -> dict:
        """Host time of the loop's parts: steps, batch rebuilds and the seconds spent in them and
        in batch iterations."""
        out = np.zeros(4)
        capi.check(capi.load().cycas_server_stats(self._h, capi.ptr(out)))
        return {"steps": int(out[0]), "rebuilds": int(out[1]), "rebuild_s": float(out[2]), "iterate_s": float(out[3])}

    def close(self):
        if getattr(self, "_h", None):
            capi.load().cycas_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
