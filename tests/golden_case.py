"""Loader of the committed golden fixtures of the reference's shipped 119x31 case."""
import os

import numpy as np

from minismac_gb300 import abi, inputs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def reference_inputs_dir():
    """The reference's ref/ folder (shipped xy.dat, bcmain.dat, smac2d.in) under the directory
    named by the environment variable SMAC_REFERENCE_DIR, or None when it is unset or missing."""
    root = os.environ.get("SMAC_REFERENCE_DIR", "")
    d = os.path.join(root, "ref") if root else ""
    return d if d and os.path.isdir(d) else None


MEAN_FLOW_KEYS = ("resmax", "rmax", "rhsnorm", "divmax", "cl", "cd", "cm", "jres", "kres")


def load_golden(impsch):
    z = np.load(os.path.join(GOLDEN, f"shipped_119x31_impsch{impsch}.npz"))
    jmax, kmax = int(z["jmax"]), int(z["kmax"])
    grid = inputs.Grid(jmax, kmax, z["x"].reshape(kmax, jmax), z["y"].reshape(kmax, jmax))
    rows = [inputs.BCRow(*[int(v) for v in r]) for r in z["bc"]]
    p = abi.default_params()
    for name, val in zip(z["param_names"], z["param_values"]):
        ctype = dict(abi.SmacParams._fields_)[str(name)]
        setattr(p, str(name), int(val) if ctype is abi.C.c_int else float(val))
    return z, grid, rows, p
