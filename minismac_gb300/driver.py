"""Host loop of the reference's main program for one subgrid on the GPU.

Mirrors ``solve`` and ``iterout`` of ref/smac2d.f:1178-1431,1667-2003: read the namelist
(smac2d.in), the grid (xy.dat) and the boundary conditions (bcmain.dat), take ntmax pseudo-time
iterations through the C ABI, print the ``XX`` convergence line of every iteration, and at the
end print the airfoil summary and write the YAML summary and, if the namelist asks for it,
Q2D.p3d.  Every iteration's residual and force scalars come back from the device with the step.

    python -m minismac_gb300.driver smac2d.in [--xy FILE] [--bcmain FILE] [--ntmax N] [--outdir DIR]
"""
from __future__ import annotations

import argparse
import os
import sys
import time

from minismac_gb300 import abi, inputs, output


def resolve(nl: dict, key_dir: str, key_file: str, override: str | None, base: str) -> str:
    if override:
        return override
    name = str(nl.get(key_file, "")).strip()
    d = str(nl.get(key_dir, "")).strip()
    for cand in (os.path.join(d, name) if d else None, os.path.join(base, name), name):
        if cand and os.path.isfile(cand):
            return cand
    raise FileNotFoundError(f"{key_file}={name!r} not found (directory {d!r}); pass it explicitly")


def run(argv=None, stdout=sys.stdout) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("namelist", help="smac2d.in")
    ap.add_argument("--xy", help="grid file (default: the namelist's xygrid_directory/xygrid_filename)")
    ap.add_argument("--bcmain", help="BC file (default: the namelist's bcmain_directory/bcmain_filename)")
    ap.add_argument("--ntmax", type=int, help="override the namelist's ntmax")
    ap.add_argument("--outdir", default=".", help="where the YAML summary and Q2D.p3d go")
    ap.add_argument("--line-solver", type=int, default=abi.LINES_PARTITIONED,
                    help="0 partitioned line solves (default), 1 sequential (reference arithmetic order)")
    a = ap.parse_args(argv)

    from minismac_gb300.solver import Solver  # fails loudly without the CUDA library

    t0 = time.perf_counter()
    nl = inputs.read_namelist(a.namelist)
    base = os.path.dirname(os.path.abspath(a.namelist))
    xy_path = resolve(nl, "xygrid_directory", "xygrid_filename", a.xy, base)
    bc_path = resolve(nl, "bcmain_directory", "bcmain_filename", a.bcmain, base)
    grid = inputs.read_xy(xy_path)
    rows = inputs.read_bcmain(bc_path)
    p = abi.params_from_namelist(nl, line_solver=a.line_solver)
    ntmax = a.ntmax if a.ntmax is not None else int(nl.get("ntmax", 200))
    solver = Solver(p, grid, rows)
    init_sec = time.perf_counter() - t0

    t1 = time.perf_counter()
    last = None
    for nt in range(1, ntmax + 1):
        h = solver.step()
        if output.xx_header_due(nt):
            print(output.XX_HEADER, file=stdout)
        print(output.xx_line(nt, h.rmax, h.divmax, h.turres, h.jres, h.kres, 1, time.perf_counter() - t1,
                             h.cd, h.cl), file=stdout)
        last = h
    solve_sec = time.perf_counter() - t1

    print("\n**************************************************", file=stdout)
    print(" summary_of_results:alpha,re,cd,cl,cm: " + output.fortran_f(p.alpha, 10, 2) +
          output.fortran_e(p.reynum, 12, 4, scale=0) +
          "".join(output.fortran_e(v, 14, 6, scale=0) for v in (last.cd, last.cl, last.cm)),
          file=stdout)
    os.makedirs(a.outdir, exist_ok=True)
    geometry = str(nl.get("geometry", "airfoil"))
    yname = output.yaml_filename(geometry, grid.jmax, grid.kmax, ntmax)
    with open(os.path.join(a.outdir, yname), "w") as fh:
        fh.write(output.yaml_summary(
            title=str(nl.get("title", "")), geometry=geometry, grid_file=os.path.basename(xy_path),
            jmax=grid.jmax, kmax=grid.kmax, beta=p.beta, dtau=p.dtau, reynum=p.reynum, alpha=p.alpha,
            impsch=p.impsch, cd=last.cd, cl=last.cl, cm=last.cm, rmax=last.rmax, ntmax=ntmax,
            init_sec=init_sec, solve_sec=solve_sec, filename=yname))
    if bool(nl.get("write_plot3d_q_file", False)):
        q = solver.get("q")
        output.write_q2d(os.path.join(a.outdir, "Q2D.p3d"), q, grid.jmax, grid.kmax, p.alpha, p.reynum, solve_sec)
    solver.close()
    return {"yaml": os.path.join(a.outdir, yname), "last": last, "solve_sec": solve_sec, "ntmax": ntmax}


if __name__ == "__main__":
    run()
