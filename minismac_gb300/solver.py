"""Host-side mirror of the reference solver's interfaces over the GB300 C ABI.

``Solver`` owns one ``smac_ctx`` (one subgrid resident on the GPU) and exposes the reference
routines under their own names: ``step`` (ref/step.f:53, plus iterout's forces), ``lrelax``
(ref/lrelax.f:51), ``lreltur`` (ref/lreltur.f:52) and ``lusgs`` (ref/lusgs.f:51), with the
reference's array arguments in Fortran order.  The library must have been built
(``minismac_gb300.build.build()``); there is no CPU fallback: without the CUDA library or a
GPU every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .build import LIB

_lib = None


class SmacError(RuntimeError):
    pass


def lib():
    """Load libsmac_gb300.so (in-tree build) and declare its C ABI."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise SmacError(f"{LIB} is missing: run minismac_gb300.build.build() first")
        L = C.CDLL(LIB)
        P = C.POINTER
        D = P(C.c_double)
        V = C.c_void_p
        L.smac_params_default.argtypes = [P(abi.SmacParams)]
        L.smac_ctx_create.argtypes = [P(abi.SmacParams), C.c_int, C.c_int, D, D, P(abi.SmacBCSpec), P(V)]
        L.smac_ctx_destroy.argtypes = [V]
        L.smac_step.argtypes = [V, P(abi.SmacIterOut)]
        L.smac_assemble.argtypes = [V, P(abi.SmacIterOut)]
        L.smac_run.argtypes = [V, C.c_int, P(abi.SmacIterOut)]
        L.smac_get_field.argtypes = [V, C.c_int, D]
        L.smac_set_field.argtypes = [V, C.c_int, D]
        L.smac_get_state.argtypes = [V, D, D, D]
        L.smac_set_state.argtypes = [V, D, D]
        L.smac_lrelax.argtypes = [V, C.c_int, C.c_int] + [D] * 8
        L.smac_lreltur.argtypes = [V, C.c_int, C.c_int] + [D] * 8
        L.smac_lusgs.argtypes = [V, C.c_int, C.c_int, C.c_int] + [D] * 9
        L.smac_last_run_ms.argtypes = [V]
        L.smac_last_run_ms.restype = C.c_double
        L.smac_launches_per_iter.argtypes = [V]
        L.smac_profile_iteration.argtypes = [V, D]
        L.smac_last_error.restype = C.c_char_p
        L.smac_autotune.argtypes = [V, P(C.c_int)]
        L.smac_assembly_tiles.argtypes = [V, P(C.c_int)]
        L.smac_batch_create.argtypes = [C.c_int, P(V), P(V)]
        L.smac_batch_run.argtypes = [V, C.c_int, P(abi.SmacIterOut)]
        L.smac_batch_last_run_ms.argtypes = [V]
        L.smac_batch_last_run_ms.restype = C.c_double
        L.smac_batch_destroy.argtypes = [V]
        L.smac_batch_options.argtypes = [V, C.c_int, C.c_int]
        L.smac_resid_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int,
                                         C.c_void_p, P(abi.SmacIterOut)]
        L.smac_noalloc_last_error.restype = C.c_char_p
        L.smac_get_clift.argtypes = [V, D]
        L.smac_set_clift.argtypes = [V, C.c_double]
        L.smac_adjoint_prepare.argtypes = [V]
        L.smac_adjoint_options.argtypes = [V, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]
        L.smac_adjoint_solve.argtypes = [V, C.c_int, C.c_double, C.c_int, P(C.c_int), D]
        L.smac_adjoint_gradient.argtypes = [V, C.c_int, C.c_int, D, D, D, D]
        L.smac_adjoint_residual.argtypes = [V, D]
        L.smac_adjoint_jacvec.argtypes = [V, C.c_int, D, D]
        L.smac_adjoint_get.argtypes = [V, C.c_int, D]
        L.smac_adjoint_forces.argtypes = [V, D, D]
        _lib = L
    return _lib


def _check(rc, what):
    if rc != abi.OK:
        raise SmacError(f"{what} failed ({rc}): {lib().smac_last_error().decode()}")


class Solver:
    """One subgrid on the GPU.  ``grid`` is an ``inputs.Grid``; ``bc_rows`` bcmain.dat rows."""

    def __init__(self, params: abi.SmacParams, grid, bc_rows):
        self.jmax, self.kmax = grid.jmax, grid.kmax
        self.N = self.jmax * self.kmax
        x, y = grid.flat()
        self._p = params
        self._bc = abi.bcspec_from_rows(bc_rows)
        h = C.c_void_p()
        _check(lib().smac_ctx_create(C.byref(self._p), self.jmax, self.kmax, abi.dptr(x), abi.dptr(y),
                                     C.byref(self._bc), C.byref(h)), "smac_ctx_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().smac_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self) -> abi.SmacIterOut:
        out = abi.SmacIterOut()
        _check(lib().smac_step(self.h, C.byref(out)), "smac_step")
        return out

    def stage_assemble(self) -> abi.SmacIterOut:
        out = abi.SmacIterOut()
        _check(lib().smac_assemble(self.h, C.byref(out)), "smac_assemble")
        return out

    def run(self, n: int) -> dict:
        hist = (abi.SmacIterOut * n)()
        _check(lib().smac_run(self.h, n, hist), "smac_run")
        return abi.hist_to_dict(hist)

    def last_run_ms(self) -> float:
        return lib().smac_last_run_ms(self.h)

    def launches_per_iter(self) -> int:
        return int(lib().smac_launches_per_iter(self.h))

    STAGES = ["sa", "assemble", "resid", "factor_j", "sweep_j", "undo_j", "factor_k", "sweep_k", "update"]

    def profile_iteration(self) -> dict:
        """Run one iteration with events at the stage boundaries; device ms per stage."""
        ms = np.zeros(len(self.STAGES))
        _check(lib().smac_profile_iteration(self.h, abi.dptr(ms)), "smac_profile_iteration")
        return dict(zip(self.STAGES, ms.tolist()))

    def autotune(self) -> tuple:
        """Lines per warp chosen for the zebra line solves (j lines, k lines)."""
        out = (C.c_int * 2)()
        _check(lib().smac_autotune(self.h, out), "smac_autotune")
        return out[0], out[1]

    def assembly_tiles(self) -> tuple:
        """Tile shapes (0..3) of the assembly kernels in use (j direction, k direction)."""
        out = (C.c_int * 2)()
        _check(lib().smac_assembly_tiles(self.h, out), "smac_assembly_tiles")
        return out[0], out[1]

    def set_state(self, q=None, turvar=None):
        qp = abi.dptr(np.ascontiguousarray(q, dtype=np.float64)) if q is not None else None
        tp = abi.dptr(np.ascontiguousarray(turvar, dtype=np.float64)) if turvar is not None else None
        _check(lib().smac_set_state(self.h, qp, tp), "smac_set_state")

    def get_state(self, q=None, turvar=None, vnut=None):
        ptr = [abi.dptr(a) if a is not None else None for a in (q, turvar, vnut)]
        _check(lib().smac_get_state(self.h, *ptr), "smac_get_state")

    def get(self, name: str) -> np.ndarray:
        f = abi.FIELD_NAMES[name]
        a = np.empty(abi.FIELD_NCOMP[f] * self.N)
        _check(lib().smac_get_field(self.h, f, abi.dptr(a)), "smac_get_field")
        return a

    def set(self, name: str, a) -> None:
        f = abi.FIELD_NAMES[name]
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != abi.FIELD_NCOMP[f] * self.N:
            raise ValueError("size mismatch")
        _check(lib().smac_set_field(self.h, f, abi.dptr(a)), "smac_set_field")

    # reference stage interfaces (arrays in/out, Fortran order)
    def lrelax(self, q, dq, s, btc, bjm, bjp, bkm, bkp):
        _check(lib().smac_lrelax(self.h, self.jmax, self.kmax,
                                 *[abi.dptr(a) for a in (q, dq, s, btc, bjm, bjp, bkm, bkp)]), "smac_lrelax")

    def lreltur(self, turvar, ds, rhs, sjm, sjp, skm, skp, stc):
        _check(lib().smac_lreltur(self.h, self.jmax, self.kmax,
                                  *[abi.dptr(a) for a in (turvar, ds, rhs, sjm, sjp, skm, skp, stc)]), "smac_lreltur")

    def lusgs(self, neqs, q, dq, rhs, btc, bjm, bjp, bkm, bkp, scr1):
        _check(lib().smac_lusgs(self.h, self.jmax, self.kmax, neqs,
                                *[abi.dptr(a) for a in (q, dq, rhs, btc, bjm, bjp, bkm, bkp, scr1)]), "smac_lusgs")

    # far-field vortex strength (restarts from a saved state)
    def get_clift(self) -> float:
        v = C.c_double()
        _check(lib().smac_get_clift(self.h, C.byref(v)), "smac_get_clift")
        return v.value

    def set_clift(self, clift: float) -> None:
        _check(lib().smac_set_clift(self.h, float(clift)), "smac_set_clift")

    # discrete adjoint (smac_adjoint_*): objectives "cl" / "cd"
    OBJECTIVES = {"cl": abi.OBJ_CL, "cd": abi.OBJ_CD}

    def adjoint_prepare(self) -> None:
        """Linearise the steady equations at the current (converged) state."""
        _check(lib().smac_adjoint_prepare(self.h), "smac_adjoint_prepare")

    def adjoint_options(self, preconditioner: str = "lines_f32", dtau: float = 0.0, inner: int = 16, sweeps: int = 1,
                        restart: int = 100) -> None:
        """Preconditioner of the transposed solve: "lines_f32" / "lines" (zebra line relaxation of
        the transposed implicit operator in FP32 / FP64) or "lusgs"; takes effect at the next
        adjoint_prepare."""
        pc = {"lusgs": 0, "lines": 1, "lines_f32": 2}[preconditioner]
        _check(lib().smac_adjoint_options(self.h, pc, dtau, inner, sweeps, restart), "smac_adjoint_options")

    def adjoint_solve(self, objective: str = "cl", rtol: float = 1e-10, max_iter: int = 2000) -> dict:
        it = C.c_int()
        rel = C.c_double()
        _check(lib().smac_adjoint_solve(self.h, self.OBJECTIVES[objective], rtol, max_iter, C.byref(it),
                                        C.byref(rel)), "smac_adjoint_solve")
        return {"iterations": it.value, "rel_resid": rel.value}

    def adjoint_gradient(self, objective: str, dxdb=None, dydb=None, dalpha=None) -> np.ndarray:
        """dJ/db of the solved objective for design variables given as grid motions (ndv x N
        arrays, j fastest) and changes of alpha in degrees (ndv values)."""
        arrs = [a for a in (dxdb, dydb) if a is not None]
        ndv = (np.atleast_2d(arrs[0]).shape[0] if arrs else len(np.atleast_1d(dalpha)))

        def prep(a, shape):
            if a is None:
                return None
            a = np.ascontiguousarray(np.reshape(a, shape), dtype=np.float64)
            return a

        dx = prep(dxdb, (ndv, self.N))
        dy = prep(dydb, (ndv, self.N))
        da = prep(dalpha, (ndv,))
        g = np.zeros(ndv)
        _check(lib().smac_adjoint_gradient(self.h, self.OBJECTIVES[objective], ndv,
                                           abi.dptr(dx) if dx is not None else None,
                                           abi.dptr(dy) if dy is not None else None,
                                           abi.dptr(da) if da is not None else None, abi.dptr(g)),
               "smac_adjoint_gradient")
        return g

    def adjoint_residual(self) -> np.ndarray:
        F = np.zeros(3 * self.N)
        _check(lib().smac_adjoint_residual(self.h, abi.dptr(F)), "smac_adjoint_residual")
        return F

    def adjoint_jacvec(self, v, transpose: bool = False) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.float64)
        y = np.zeros(3 * self.N)
        _check(lib().smac_adjoint_jacvec(self.h, int(transpose), abi.dptr(v), abi.dptr(y)), "smac_adjoint_jacvec")
        return y

    def adjoint_get(self, name: str) -> np.ndarray:
        f = abi.ADJ_FIELDS[name]
        n = 81 * self.N if name == "jacobian" else 3 * self.N
        a = np.zeros(n)
        _check(lib().smac_adjoint_get(self.h, f, abi.dptr(a)), "smac_adjoint_get")
        return a

    def adjoint_forces(self) -> tuple:
        cl, cd = C.c_double(), C.c_double()
        _check(lib().smac_adjoint_forces(self.h, C.byref(cl), C.byref(cd)), "smac_adjoint_forces")
        return cl.value, cd.value


class Batch:
    """Independent cases advanced together: one CUDA graph launch per iteration of all of them
    (smac_batch_*).  The solvers stay owned by the caller and must outlive the batch."""

    def __init__(self, solvers, packed: bool = False, warps_per_line: int = 2, queue: bool = False):
        """packed: the line solves of all cases in one launch per sweep colour
        (smac_batch_options, SMAC_BATCH_PACKED_LINES); queue: the line sweeps of an iteration of
        all cases in one persistent launch fed by one work queue (SMAC_BATCH_QUEUE_LINES)."""
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = C.c_void_p()
        _check(lib().smac_batch_create(len(self.solvers), arr, C.byref(h)), "smac_batch_create")
        self.h = h.value
        if queue:
            _check(lib().smac_batch_options(self.h, abi.BATCH_QUEUE_LINES, warps_per_line), "smac_batch_options")
        elif packed:
            _check(lib().smac_batch_options(self.h, abi.BATCH_PACKED_LINES, warps_per_line), "smac_batch_options")

    def close(self):
        if getattr(self, "h", None):
            lib().smac_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, n: int) -> list:
        """n iterations of every case; a history dict per case."""
        hist = (abi.SmacIterOut * (n * len(self.solvers)))()
        _check(lib().smac_batch_run(self.h, n, hist), "smac_batch_run")
        return [abi.hist_to_dict(hist[k * n:(k + 1) * n]) for k in range(len(self.solvers))]

    def last_run_ms(self) -> float:
        return lib().smac_batch_last_run_ms(self.h)
