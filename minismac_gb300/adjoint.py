"""Gradients of Cl and Cd through the discrete adjoint of the converged iteration.

``gradients`` linearises a converged ``Solver`` (smac_adjoint_prepare), solves the transposed
system for each objective (smac_adjoint_solve) and returns dJ/db for the variables of a
``design.Design`` (smac_adjoint_gradient).  ``converge`` runs a solver to its round-off floor;
``finite_differences`` gives the central differences of the same variables by re-converging
solvers on moved grids, warm-started from the base state (the check of the adjoint).
"""
from __future__ import annotations

import time

import numpy as np


def converge(s, max_iter: int = 60000, chunk: int = 1000, tol_cl: float = 1e-15) -> dict:
    """Iterate until the residual stops falling and Cl stops moving (round-off floor) or
    max_iter iterations.  Returns the iteration count, the last resmax, Cl, Cd."""
    n = 0
    best = np.inf
    stall = 0
    cl_prev = None
    h = None
    while n < max_iter:
        h = s.run(chunk)
        n += chunk
        r = float(np.min(h["resmax"]))
        cl = float(h["cl"][-1])
        moved = cl_prev is None or abs(cl - cl_prev) > tol_cl
        stall = stall + 1 if r > 0.5 * best else 0
        best = min(best, r)
        cl_prev = cl
        if stall >= 2 and not moved:
            break
    return {"iterations": n, "resmax": float(h["resmax"][-1]), "cl": float(h["cl"][-1]),
            "cd": float(h["cd"][-1])}


def gradients(s, design, objectives=("cl", "cd"), rtol: float = 1e-11, max_iter: int = 4000,
              names=None) -> dict:
    """Adjoint gradients at the solver's (converged) state: {objective: array over names}, plus
    the solve statistics and timings."""
    names = design.names if names is None else list(names)
    out = {"names": names, "stats": {}}
    t0 = time.perf_counter()
    s.adjoint_prepare()
    out["prepare_s"] = time.perf_counter() - t0
    dxdb, dydb, da = design.sensitivities(names)
    for obj in objectives:
        t1 = time.perf_counter()
        st = s.adjoint_solve(obj, rtol, max_iter)
        t2 = time.perf_counter()
        out[obj] = s.adjoint_gradient(obj, dxdb, dydb, da)
        st["solve_s"] = t2 - t1
        st["gradient_s"] = time.perf_counter() - t2
        out["stats"][obj] = st
    return out


def finite_differences(make_solver, design, names, h: float, q0, clift0: float, **conv) -> dict:
    """Central differences (J(+h) - J(-h)) / 2h of Cl and Cd for each variable.
    make_solver(grid, dalpha) returns a solver for that grid and angle change; each starts from
    the state q0 and far-field vortex clift0 and is converged with ``converge``."""
    res = {"cl": [], "cd": [], "iterations": []}
    for name in names:
        vals = []
        for sgn in (1.0, -1.0):
            grid, dalpha = design.moved(name, sgn * h)
            s = make_solver(grid, dalpha)
            s.set_state(q=q0)
            s.set_clift(clift0)
            c = converge(s, **conv)
            vals.append(c)
            res["iterations"].append(c["iterations"])
            if hasattr(s, "close"):
                s.close()
        res["cl"].append((vals[0]["cl"] - vals[1]["cl"]) / (2 * h))
        res["cd"].append((vals[0]["cd"] - vals[1]["cd"]) / (2 * h))
    res["cl"] = np.array(res["cl"])
    res["cd"] = np.array(res["cd"])
    return res


def main(argv=None) -> int:
    """python -m minismac_gb300.adjoint [--grid 481x121] [--iters N] [--max-gmres M]: gradients of
    Cl and Cd for alpha and 16 Hicks-Henne bumps on a NACA 4412 C-grid (laminar Re = 1000),
    after converging the flow (or after N iterations when --iters is given), as one JSON line."""
    import argparse
    import json

    from . import abi, design, inputs
    from .solver import Solver
    ap = argparse.ArgumentParser(prog="python -m minismac_gb300.adjoint")
    ap.add_argument("--grid", default="481x121")
    ap.add_argument("--alpha", type=float, default=5.0)
    ap.add_argument("--reynum", type=float, default=1000.0)
    ap.add_argument("--iters", type=int, default=0, help="primal iterations (0: converge to the floor)")
    ap.add_argument("--max-gmres", type=int, default=6000)
    ap.add_argument("--rtol", type=float, default=1e-11)
    a = ap.parse_args(argv)
    jm, km = (int(v) for v in a.grid.split("x"))
    g, rows = inputs.naca4_cgrid(jm, km)
    p = abi.default_params(alpha=a.alpha, beta=10.0, reynum=a.reynum, dtau=0.5, underr=1.0, impsch=1, iturb=0,
                           visc_fp64=1, precision=abi.PREC_MIXED, order=abi.ORDER_MULTICOLOR)
    s = Solver(p, g, rows)
    if a.iters > 0:
        h = s.run(a.iters)
        primal = {"iterations": a.iters, "resmax": float(h["resmax"][-1])}
    else:
        primal = converge(s)
    d = design.Design(g, rows)
    r = gradients(s, d, rtol=a.rtol, max_iter=a.max_gmres)
    print(json.dumps({"grid": a.grid, "primal": primal, "names": d.names, "cl": r["cl"].tolist(),
                      "cd": r["cd"].tolist(), "solve": r["stats"]}))
    s.close()
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(main())
