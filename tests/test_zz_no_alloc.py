"""The allocation-free residual entry point (smac_resid_noalloc).

It serves callers that cannot call cudaMalloc (a host that owns all device memory itself,
or runs under a fixed device-memory budget): its scratch is a fixed file-scope device array.
Here the test plays such a caller: it owns the device copies of s and dj, and checks two
consecutive calls against the residual scalars the context-based entry point (smac_assemble)
reports for the same fields.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from minismac_gb300 import abi, inputs

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.fail("libcudart not found")


class DeviceArray:
    """A device buffer owned by the caller (the test), not by the library."""

    def __init__(self, rt, host: np.ndarray):
        self.rt = rt
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.ptr), ctypes.c_size_t(host.nbytes)) == 0
        assert rt.cudaMemcpy(self.ptr, host.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(host.nbytes), 1) == 0

    def free(self):
        if self.ptr:
            self.rt.cudaFree(self.ptr)
            self.ptr = None


def test_resid_noalloc_matches_context_entry_point(cuda_lib):
    from minismac_gb300.solver import Solver, lib
    g, rows = inputs.naca4_cgrid(119, 31)
    beta = 10.0
    s = Solver(abi.default_params(alpha=5.0, beta=beta, reynum=1e6), g, rows)
    ref = s.stage_assemble()          # the context-based entry point, iteration 1
    s_host, dj_host = s.get("s"), s.get("dj")
    rt = _cudart()
    d_s, d_dj = DeviceArray(rt, s_host), DeviceArray(rt, dj_host)
    try:
        for call in range(2):         # two calls in a row share the static scratch
            out = abi.SmacIterOut()
            rc = lib().smac_resid_noalloc(d_s.ptr, d_dj.ptr, g.jmax, g.kmax, beta, 1, None, ctypes.byref(out))
            assert rc == 0, lib().smac_noalloc_last_error().decode()
            assert (out.jres, out.kres, out.neq_res) == (ref.jres, ref.kres, ref.neq_res), call
            assert out.resmax == ref.resmax and out.resmax0 == ref.resmax0, call
            assert out.divmax == ref.divmax, call
            assert abs(out.rhsnorm - ref.rhsnorm) <= 1e-13 * ref.rhsnorm, call
        # a later iteration: the same residual scalars, and no resmax0 kept between calls, so
        # resmax0, rmax and nt come back as 0
        out = abi.SmacIterOut()
        rc = lib().smac_resid_noalloc(d_s.ptr, d_dj.ptr, g.jmax, g.kmax, beta, 0, None, ctypes.byref(out))
        assert rc == 0, lib().smac_noalloc_last_error().decode()
        assert (out.jres, out.kres, out.neq_res) == (ref.jres, ref.kres, ref.neq_res)
        assert out.resmax == ref.resmax and out.divmax == ref.divmax
        assert out.resmax0 == 0.0 and out.rmax == 0.0 and out.nt == 0
        # a warm call takes no device memory: the free bytes the driver reports do not move
        free0, free1, total = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
        assert rt.cudaMemGetInfo(ctypes.byref(free0), ctypes.byref(total)) == 0
        out = abi.SmacIterOut()
        rc = lib().smac_resid_noalloc(d_s.ptr, d_dj.ptr, g.jmax, g.kmax, beta, 1, None, ctypes.byref(out))
        assert rc == 0 and out.resmax == ref.resmax
        assert rt.cudaMemGetInfo(ctypes.byref(free1), ctypes.byref(total)) == 0
        assert free1.value == free0.value, (free0.value, free1.value)
        # sizes beyond the stated maximum are rejected
        out = abi.SmacIterOut()
        rc = lib().smac_resid_noalloc(d_s.ptr, d_dj.ptr, 9000, 31, beta, 1, None, ctypes.byref(out))
        assert rc == abi.ERR_ARG and b"8100" in lib().smac_noalloc_last_error()
        # a call on a stream that is being captured is refused before it touches the stream
        # (its host copies and synchronisation would invalidate the capture); the capture
        # then ends normally with an empty graph
        st, graph = ctypes.c_void_p(), ctypes.c_void_p()
        assert rt.cudaStreamCreate(ctypes.byref(st)) == 0
        try:
            assert rt.cudaStreamBeginCapture(st, 2) == 0      # cudaStreamCaptureModeRelaxed
            out = abi.SmacIterOut()
            rc = lib().smac_resid_noalloc(d_s.ptr, d_dj.ptr, g.jmax, g.kmax, beta, 1, st, ctypes.byref(out))
            assert rt.cudaStreamEndCapture(st, ctypes.byref(graph)) == 0
            assert rc == abi.ERR_UNSUPPORTED and b"captured" in lib().smac_noalloc_last_error()
            assert rt.cudaGraphDestroy(graph) == 0
        finally:
            rt.cudaStreamDestroy(st)
        out = abi.SmacIterOut()
        rc = lib().smac_resid_noalloc(d_s.ptr, d_dj.ptr, g.jmax, g.kmax, beta, 1, None, ctypes.byref(out))
        assert rc == 0 and out.resmax == ref.resmax
    finally:
        d_s.free()
        d_dj.free()
        s.close()
