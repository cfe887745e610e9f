"""Record the long comparison of the GPU path with the oracle at 481x121.

The workload family's second configuration: the NACA 4412 C-grid scaled to 481x121, alpha 5
degrees, Re 1e6, beta 10, dtau 0.1, underr 0.01, 5000 pseudo-time iterations, line relaxation
(impsch 1) and LU-SGS (impsch 2), the plain FP64 GPU path (reference line order, partitioned
line solves) against the oracle on the same inputs.  The GPU runs in this process, the oracle
(all host threads) in a spawned one beside it.

Writes parity_481x121_5000.json next to this script: for each scheme the largest deviation
over the whole history of the per-iteration L2 residual (rhsnorm, relative), of resmax
(relative), of Cl and Cd (relative to their largest magnitude), the number of iterations whose
resmax location differs, the final p, u, v deviation (relative to the largest |q|), the same
figures at every 500th iteration, and both runs' final Cl, Cd and rmax.
tests/test_parity_record.py checks the committed record against the tolerances.

Usage (needs a GPU and the built library):  python tests/golden/record_parity_481x121.py [ITERS]
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

GRID = (481, 121)
OUT = os.path.join(HERE, "parity_481x121_5000.json")
KEYS = ("rhsnorm", "resmax", "cl", "cd", "jres", "kres", "rmax")


def params(impsch):
    from minismac_gb300 import abi
    return abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, dtau=0.1, underr=0.01, impsch=impsch)


def oracle_run(args):
    sys.path.insert(0, ROOT)
    from minismac_gb300 import inputs
    from oracle.oracle_py import Oracle
    impsch, n = args
    g, rows = inputs.naca4_cgrid(*GRID)
    o = Oracle(params(impsch), g, rows)
    o.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    h = o.run(n)
    dt = time.perf_counter() - t0
    out = {k: h[k] for k in KEYS}
    out["q"] = o.get("q")
    out["seconds"] = dt
    o.close()
    return out


def deviations(hg, ho, upto):
    s = slice(0, upto)
    return {
        "rhsnorm_rel": float(np.max(np.abs(hg["rhsnorm"][s] / ho["rhsnorm"][s] - 1.0))),
        "resmax_rel": float(np.max(np.abs(hg["resmax"][s] / ho["resmax"][s] - 1.0))),
        "cl_rel": float(np.max(np.abs(hg["cl"][s] - ho["cl"][s])) / np.abs(ho["cl"][s]).max()),
        "cd_rel": float(np.max(np.abs(hg["cd"][s] - ho["cd"][s])) / np.abs(ho["cd"][s]).max()),
        "resmax_location_mismatches": int(np.sum((hg["jres"][s] != ho["jres"][s]) | (hg["kres"][s] != ho["kres"][s]))),
    }


def main(argv):
    from minismac_gb300 import build, inputs
    from minismac_gb300.solver import Solver
    n = int(argv[1]) if len(argv) > 1 else 5000
    build.build()
    g, rows = inputs.naca4_cgrid(*GRID)
    record = {"workload": f"NACA 4412 C-grid {GRID[0]}x{GRID[1]}, alpha 5, Re 1e6, beta 10, dtau 0.1, "
                          "underr 0.01; plain FP64 GPU path (reference line order, partitioned line solves) "
                          "against the oracle (all host threads)",
              "iterations": n, "schemes": {}}
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        for impsch in (1, 2):
            fut = pool.apply_async(oracle_run, ((impsch, n),))
            s = Solver(params(impsch), g, rows)
            t0 = time.perf_counter()
            hg = s.run(n)
            gpu_s = time.perf_counter() - t0
            qg = s.get("q")
            s.close()
            ho = fut.get()
            d = deviations(hg, ho, n)
            d["q_final_rel"] = float(np.abs(qg - ho["q"]).max() / np.abs(ho["q"]).max())
            d["checkpoints"] = {str(i): deviations(hg, ho, i) for i in range(500, n + 1, 500)}
            d["final"] = {"gpu": {k: float(hg[k][-1]) for k in ("cl", "cd", "rmax")},
                          "oracle": {k: float(ho[k][-1]) for k in ("cl", "cd", "rmax")}}
            d["seconds"] = {"gpu_wall": gpu_s, "oracle_wall": ho["seconds"]}
            record["schemes"]["line relaxation" if impsch == 1 else "LU-SGS"] = d
            print(impsch, {k: v for k, v in d.items() if k != "checkpoints"}, flush=True)
    with open(OUT, "w") as fh:
        json.dump(record, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv)
