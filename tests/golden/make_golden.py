"""Generate the golden fixtures of the 119x31 case that ships with the reference.

Reads the reference's own input files (ref/xy.dat_original_119x31,
ref/bcmain.dat_original_119x31, ref/smac2d.in) from the reference checkout, runs the CPU
oracle on them for the namelist's ntmax = 200 pseudo-time iterations with line relaxation
(impsch 1) and with LU-SGS (impsch 2), and writes one compressed .npz per scheme holding

  - the grid (x, y) and BC rows, so that a test can rebuild the case without the reference,
  - the flow parameters used,
  - the per-iteration history (resmax, rmax, rhsnorm, divmax, turres, cl, cd, cm, jres, kres),
  - the final p, u, v, anut fields.

The reference itself cannot be built here (no Fortran compiler), so these vectors pin the
oracle against regressions and carry the shipped inputs to machines without the reference.

Usage:  python tests/golden/make_golden.py [REFERENCE_ROOT]   (or SMAC_REFERENCE_DIR=REFERENCE_ROOT)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from minismac_gb300 import abi, inputs  # noqa: E402
from oracle.oracle_py import Oracle  # noqa: E402

HIST_KEYS = ("resmax", "rmax", "rhsnorm", "divmax", "turres", "cl", "cd", "cm", "jres", "kres")


def shipped_case(ref_root: str):
    d = os.path.join(ref_root, "ref")
    grid = inputs.read_xy(os.path.join(d, "xy.dat_original_119x31"))
    rows = inputs.read_bcmain(os.path.join(d, "bcmain.dat_original_119x31"))
    nl = inputs.read_namelist(os.path.join(d, "smac2d.in"))
    return grid, rows, nl


def run_case(grid, rows, nl, impsch: int, n: int):
    p = abi.params_from_namelist(nl, impsch=impsch)
    o = Oracle(p, grid, rows)
    h = o.run(n)
    fields = {"q": o.get("q"), "anut": o.get("anut")}
    o.close()
    return p, h, fields


def main(argv):
    ref_root = argv[1] if len(argv) > 1 else os.environ.get("SMAC_REFERENCE_DIR", "")
    if not ref_root:
        raise SystemExit("usage: make_golden.py REFERENCE_DIR (or set SMAC_REFERENCE_DIR)")
    grid, rows, nl = shipped_case(ref_root)
    n = int(nl.get("ntmax", 200))
    x, y = grid.flat()
    bc = np.array([[r.ibcval, r.zone, r.jbeg, r.jend, r.kbeg, r.kend] for r in rows], dtype=np.int64)
    for impsch in (1, 2):
        p, h, f = run_case(grid, rows, nl, impsch, n)
        par = {k: getattr(p, k) for k, _ in abi.SmacParams._fields_ if k != "reserved"}
        out = os.path.join(HERE, f"shipped_119x31_impsch{impsch}.npz")
        np.savez_compressed(
            out, jmax=grid.jmax, kmax=grid.kmax, x=x, y=y, bc=bc,
            param_names=np.array(list(par.keys())), param_values=np.array([float(v) for v in par.values()]),
            **{f"hist_{k}": np.asarray(h[k]) for k in HIST_KEYS}, q=f["q"], anut=f["anut"])
        print(f"wrote {out}: {n} iterations, rmax[-1]={h['rmax'][-1]:.3e} cl[-1]={h['cl'][-1]:.6f}")


if __name__ == "__main__":
    main(sys.argv)
