"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, and
only as the checker / the timed CPU reference: the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from minismac_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsmac_oracle.so")
SRC = os.path.join(HERE, "smac_oracle.c")
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-fopenmp", "-shared", "-fPIC"]

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, no fast-math)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", *CFLAGS, "-o", LIB, SRC, "-lm"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        D = P(C.c_double)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [P(abi.SmacParams), C.c_int, C.c_int, D, D, P(abi.SmacBCSpec)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_step.argtypes = [C.c_void_p, P(abi.SmacIterOut)]
        L.orc_run.argtypes = [C.c_void_p, C.c_int, P(abi.SmacIterOut)]
        L.orc_stage_assemble.argtypes = [C.c_void_p, P(abi.SmacIterOut)]
        L.orc_get_field.argtypes = [C.c_void_p, C.c_int, D]
        L.orc_set_field.argtypes = [C.c_void_p, C.c_int, D]
        L.orc_lrelax.argtypes = [C.c_void_p, D, D, D, D, D, D, D, D]
        L.orc_lreltur.argtypes = [C.c_void_p, D, D, D, D, D, D, D, D]
        L.orc_lusgs.argtypes = [C.c_void_p, C.c_int, D, D, D, D, D, D, D, D, D]
        L.orc_last_error.restype = C.c_char_p
        L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_get_clift.argtypes = [C.c_void_p, D]
        L.orc_set_clift.argtypes = [C.c_void_p, C.c_double]
        _lib = L
    return _lib


class Oracle:
    """One subgrid on the CPU, same interface as minismac_gb300.solver.Solver."""

    def __init__(self, params, grid, bc_rows):
        self.jmax, self.kmax = grid.jmax, grid.kmax
        self.N = self.jmax * self.kmax
        x, y = grid.flat()
        self._p = params
        self._bc = abi.bcspec_from_rows(bc_rows)
        self.h = lib().orc_create(C.byref(self._p), self.jmax, self.kmax, abi.dptr(x), abi.dptr(y),
                                  C.byref(self._bc))
        if not self.h:
            raise RuntimeError("oracle create failed: " + lib().orc_last_error().decode())

    def set_threads(self, n: int):
        """OpenMP threads on the loops the reference parallelises (1 = serial)."""
        if lib().orc_set_threads(self.h, int(n)):
            raise ValueError("thread count must be >= 1")

    def get_clift(self) -> float:
        v = C.c_double()
        lib().orc_get_clift(self.h, C.byref(v))
        return v.value

    def set_clift(self, clift: float) -> None:
        lib().orc_set_clift(self.h, float(clift))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    __del__ = close

    def step(self):
        out = abi.SmacIterOut()
        rc = lib().orc_step(self.h, C.byref(out))
        if rc:
            raise RuntimeError(f"oracle step failed ({rc})")
        return out

    def run(self, n):
        hist = (abi.SmacIterOut * n)()
        rc = lib().orc_run(self.h, n, hist)
        if rc:
            raise RuntimeError(f"oracle run failed ({rc})")
        return abi.hist_to_dict(hist)

    def stage_assemble(self):
        out = abi.SmacIterOut()
        rc = lib().orc_stage_assemble(self.h, C.byref(out))
        if rc:
            raise RuntimeError(f"oracle assemble failed ({rc})")
        return out

    def get(self, name):
        f = abi.FIELD_NAMES[name]
        a = np.empty(abi.FIELD_NCOMP[f] * self.N)
        lib().orc_get_field(self.h, f, abi.dptr(a))
        return a

    def set(self, name, a):
        f = abi.FIELD_NAMES[name]
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == abi.FIELD_NCOMP[f] * self.N
        lib().orc_set_field(self.h, f, abi.dptr(a))

    # the reference's stage interfaces on caller arrays
    def lrelax(self, q, dq, s, btc, bjm, bjp, bkm, bkp):
        lib().orc_lrelax(self.h, *[abi.dptr(a) for a in (q, dq, s, btc, bjm, bjp, bkm, bkp)])

    def lreltur(self, turvar, ds, rhs, sjm, sjp, skm, skp, stc):
        lib().orc_lreltur(self.h, *[abi.dptr(a) for a in (turvar, ds, rhs, sjm, sjp, skm, skp, stc)])

    def lusgs(self, neqs, q, dq, rhs, btc, bjm, bjp, bkm, bkp, scr1):
        rc = lib().orc_lusgs(self.h, neqs, *[abi.dptr(a) for a in (q, dq, rhs, btc, bjm, bjp, bkm, bkp, scr1)])
        if rc:
            raise RuntimeError("oracle lusgs failed")
