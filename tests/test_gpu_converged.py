"""Converged states of the GPU forms and of the oracle, on a case with a steady state: laminar
Re = 1000 on a 59x17 NACA 4412 C-grid, with the wall distance kept on every SA call
(SMAC_WALLDIST_FIXED, a labelled deviation: with the reference's quirk the SA variable collapses
and its comparison would say nothing), all run 25,000 iterations, past the round-off floor of
the mean flow.

Plain FP64 path (reference line order, partitioned line solves) against the oracle: the two
converged states agree to ~1e-8 in p, u, v, ~1e-9 relative in the SA variable and ~1e-9..3e-9 in
Cl and Cd, the width of the round-off band of a fixed point whose near-wall residual is scaled
by dj ~ 1e8 (the sequential-line GPU path is bit-identical to the oracle;
tests/test_gpu_golden.py).  The bounds below sit above those figures.

The throughput forms (zebra line order in FP64, and the FP32 implicit operator in FP64 defect
correction) have the same mean-flow fixed point, s = 0 in FP64: their converged p, u, v, Cl and
Cd are held to the same band against the oracle, each stated separately.  The SA variable is
not converged here in any form: it decays towards zero for tens of thousands of iterations more
(its largest value falls ~50x over the next 25,000), which the SA criterion, the largest
positive update (ref/tursa.f:314-347), does not see, and the decay runs at a different pace in
another line order.  So the SA variable is compared along the same path: the plain path with
the oracle, the FP32-operator form with the FP64 zebra form (the SA model stays FP64 in both).
"""
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


FORMS = {"plain FP64, reference order": {},
         "FP64, zebra order": dict(order=abi.ORDER_MULTICOLOR),
         "FP32 operator in FP64 defect correction": dict(order=abi.ORDER_MULTICOLOR, precision=abi.PREC_MIXED)}


def test_converged_state_matches_oracle(cuda_lib):
    import multiprocessing as mp
    from oracle.oracle_py import build as build_oracle
    from minismac_gb300.solver import Solver
    build_oracle()
    jm, km = 59, 17
    runs = {}
    with mp.get_context("spawn").Pool(1) as pool:
        fut = pool.apply_async(_oracle_run, ((jm, km, N_ITER),))  # CPU, beside the GPU runs
        g, rows = inputs.naca4_cgrid(jm, km)
        for name, form in FORMS.items():
            p = _params()
            for k, v in form.items():
                setattr(p, k, v)
            s = Solver(p, g, rows)
            runs[name] = (s.run(N_ITER), s.get("q"), s.get("anut"))
            s.close()
        ho = fut.get()
    assert ho["rmax"][-1] < 1e-10 and ho["turres"][-1] < 1e-10
    n = jm * km

    def rel_nu(a, b):
        return float(np.abs(a - b).max() / np.abs(b).max())

    for name, (hg, qg, ag) in runs.items():
        assert hg["rmax"][-1] < 1e-10 and hg["turres"][-1] < 1e-10, name
        d = {var: float(np.abs(qg[i * n:(i + 1) * n] - ho["q"][i * n:(i + 1) * n]).max())
             for i, var in enumerate(("p", "u", "v"))}
        d["cl"] = abs(hg["cl"][-1] - ho["cl"][-1])
        d["cd"] = abs(hg["cd"][-1] - ho["cd"][-1])
        d["nu~ rel, oracle"] = rel_nu(ag, ho["anut"])
        print(f"converged differences from the oracle, {name}:", d)
        assert max(d["p"], d["u"], d["v"]) < 5e-8, (name, d)
        assert d["cl"] < 1e-8 and d["cd"] < 1e-8, (name, d)
    # the SA variable along the same path
    assert rel_nu(runs["plain FP64, reference order"][2], ho["anut"]) < 5e-9
    dz = rel_nu(runs["FP32 operator in FP64 defect correction"][2], runs["FP64, zebra order"][2])
    print("SA variable, FP32-operator form against FP64 zebra order, relative:", dz)
    assert dz < 1e-8
