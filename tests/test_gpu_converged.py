"""Converged states of the plain FP64 GPU path (reference line order, partitioned line solves)
and of the oracle, on a case with a steady state: laminar Re = 1000 on a 59x17 NACA 4412
C-grid, with the wall distance kept on every SA call (SMAC_WALLDIST_FIXED, a labelled deviation:
with the reference's quirk the SA variable collapses and its comparison would say nothing),
both run 25,000 iterations, past the round-off floor of the mean flow and of the SA model.

Measured: the two converged states agree to ~1e-8 in p, u, v, ~1e-9 relative in the SA
variable and ~1e-9..3e-9 in Cl and Cd, the width of the round-off band of a fixed point whose
near-wall residual is scaled by dj ~ 1e8 (the sequential-line GPU path is bit-identical to the
oracle; tests/test_gpu_golden.py).  The bounds below sit above those figures."""
import numpy as np
import pytest

from minismac_gb300 import abi, inputs

pytestmark = pytest.mark.gpu

N_ITER = 25000


def _params():
    return abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0,
                              wall_distance=abi.WALLDIST_FIXED)


def _oracle_run(args):
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from minismac_gb300 import inputs as _inputs
    from oracle.oracle_py import Oracle
    jm, km, n = args
    g, rows = _inputs.naca4_cgrid(jm, km)
    o = Oracle(_params(), g, rows)
    h = o.run(n)
    out = {k: h[k] for k in ("rmax", "turres", "cl", "cd")}
    out["q"], out["anut"] = o.get("q"), o.get("anut")
    o.close()
    return out


def test_converged_state_matches_oracle(cuda_lib):
    import multiprocessing as mp
    from oracle.oracle_py import build as build_oracle
    from minismac_gb300.solver import Solver
    build_oracle()
    jm, km = 59, 17
    with mp.get_context("spawn").Pool(1) as pool:
        fut = pool.apply_async(_oracle_run, ((jm, km, N_ITER),))  # CPU, beside the GPU run
        g, rows = inputs.naca4_cgrid(jm, km)
        s = Solver(_params(), g, rows)
        hg = s.run(N_ITER)
        qg, ag = s.get("q"), s.get("anut")
        ho = fut.get()
    for h in (hg, ho):
        assert h["rmax"][-1] < 1e-10 and h["turres"][-1] < 1e-10
    dq = np.abs(qg - ho["q"]).max()
    dnu = np.abs(ag - ho["anut"]).max() / np.abs(ho["anut"]).max()
    dcl, dcd = abs(hg["cl"][-1] - ho["cl"][-1]), abs(hg["cd"][-1] - ho["cd"][-1])
    print("converged differences: q", dq, "nu~ rel", dnu, "cl", dcl, "cd", dcd)
    assert dq < 5e-8
    assert dnu < 5e-9
    assert dcl < 1e-8 and dcd < 1e-8
