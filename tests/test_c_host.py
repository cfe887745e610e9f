"""A compiled C host against include/smac_gb300.h, as the Fortran ISO_C_BINDING module uses it.

tests/host_c/smac_host.c is built with gcc from the header alone and linked to the library:
smac_params_default, smac_ctx_create, smac_step per iteration, smac_get_state and
smac_ctx_destroy.  The build runs everywhere (it checks that the header is plain C and that the
library exports what the host links); the run needs a GPU and compares the iteration history
and the final state with the oracle on the same grid, BC rows and flow.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from minismac_gb300 import abi, build, inputs

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "host_c", "smac_host.c")


def compile_host(out_dir):
    lib = build.build()
    exe = os.path.join(str(out_dir), "smac_host")
    libdir = os.path.dirname(lib)
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", libdir, "-lsmac_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def write_input(path, grid, rows, nsteps, alpha, beta, reynum):
    x, y = grid.flat()
    with open(path, "wb") as fh:
        fh.write(struct.pack("=4i3d", grid.jmax, grid.kmax, len(rows), nsteps, alpha, beta, reynum))
        for r in rows:
            fh.write(struct.pack("=6i", r.ibcval, r.zone, r.jbeg, r.jend, r.kbeg, r.kend))
        fh.write(np.ascontiguousarray(x, dtype="<f8").tobytes())
        fh.write(np.ascontiguousarray(y, dtype="<f8").tobytes())


def test_c_host_builds_against_the_header(tmp_path):
    exe = compile_host(tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_c_host_matches_oracle(cuda_lib, tmp_path):
    from oracle.oracle_py import Oracle
    exe = compile_host(tmp_path)
    g, rows = inputs.naca4_cgrid(119, 31)
    n, alpha, beta, re = 10, 5.0, 10.0, 1e6
    inp, outp = os.path.join(tmp_path, "in.bin"), os.path.join(tmp_path, "out.bin")
    write_input(inp, g, rows, n, alpha, beta, re)
    r = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    hist = np.array([[float(v) for v in line.split()] for line in r.stdout.strip().splitlines()])
    assert hist.shape == (n, 5)
    N = g.jmax * g.kmax
    raw = np.fromfile(outp, dtype="<f8")
    assert raw.size == 5 * N
    q = raw[:3 * N]
    # the host filled the parameters from smac_params_default and set the flow: the oracle runs
    # the same values from the Python mirror of the defaults
    orc = Oracle(abi.default_params(alpha=alpha, beta=beta, reynum=re), g, rows)
    ho = orc.run(n)
    qo = orc.get("q")
    np.testing.assert_array_equal(hist[:, 0], ho["nt"])
    for col, key in ((1, "cl"), (2, "cd")):
        assert np.abs(hist[:, col] - ho[key]).max() < 1e-9 * np.abs(ho[key]).max(), key
    assert np.abs(hist[:, 3] / ho["resmax"] - 1).max() < 1e-9
    assert np.abs(hist[:, 4] / ho["rhsnorm"] - 1).max() < 1e-10
    assert np.abs(q - qo).max() < 1e-9 * np.abs(qo).max()
