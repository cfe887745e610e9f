"""One pseudo-time iteration between cudaProfilerStart and cudaProfilerStop, for profilers.

Builds the bench workload (NACA 4412 C-grid, alpha 5, Re 1e6) at the given size and form,
runs the warm-up iterations (context setup, wall distance, graph capture and autotuning happen
here), then exactly one iteration inside the profiler range, so that a profiler started with
its capture range tied to the CUDA profiler API (ncu --profile-from-start off) sees the kernels
of one iteration and nothing else.

    python -m minismac_gb300.profile_iteration --jmax 961 --kmax 241 --mode reference
"""
from __future__ import annotations

import argparse
import ctypes
import os

from minismac_gb300 import abi, inputs

FORMS = {"reference": dict(order=0, precision=0), "multicolor": dict(order=1, precision=0),
         "mixed": dict(order=1, precision=1)}


def cudart():
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            pass
    lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so")
    return ctypes.CDLL(lib)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--jmax", type=int, default=1921)
    ap.add_argument("--kmax", type=int, default=481)
    ap.add_argument("--mode", default="reference", choices=sorted(FORMS))
    ap.add_argument("--impsch", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    a = ap.parse_args(argv)
    from minismac_gb300 import build
    build.build()
    from minismac_gb300.solver import Solver
    g, rows = inputs.naca4_cgrid(a.jmax, a.kmax)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1.0e6, dtau=0.1, underr=0.01, impsch=a.impsch,
                           **FORMS[a.mode])
    s = Solver(p, g, rows)
    s.run(a.warmup)
    rt = cudart()
    if rt.cudaProfilerStart() != 0:
        raise RuntimeError("cudaProfilerStart failed")
    s.run(1)
    rt.cudaProfilerStop()
    s.close()


if __name__ == "__main__":
    main()
