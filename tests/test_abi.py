"""The C-ABI library: built for sm_103a, loadable, exporting every symbol of include/*.h.
No compute call is made here (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "smac_gb300.h")).read()
    return sorted(set(re.findall(r"\b(smac_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_header_symbols():
    from minismac_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    syms = header_symbols()
    assert "smac_step" in syms and "smac_lrelax" in syms and "smac_lusgs" in syms
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_struct_sizes_match_header():
    """ctypes mirrors agree with the C struct layout (checked with the host compiler)."""
    import subprocess
    import tempfile
    from minismac_gb300 import abi
    src = r'''
#include <stdio.h>
#include "smac_gb300.h"
int main(void){printf("%zu %zu %zu\n", sizeof(smac_params), sizeof(smac_bcspec), sizeof(smac_iter_out));return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        exe = os.path.join(d, "s")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    assert [int(v) for v in out] == [ctypes.sizeof(abi.SmacParams), ctypes.sizeof(abi.SmacBCSpec),
                                     ctypes.sizeof(abi.SmacIterOut)]


def test_params_default_matches_python():
    from minismac_gb300 import abi, build
    lib = ctypes.CDLL(build.build())
    p = abi.SmacParams()
    lib.smac_params_default(ctypes.byref(p))
    q = abi.default_params()
    for f, _ in abi.SmacParams._fields_:
        if f == "reserved":
            continue
        assert getattr(p, f) == getattr(q, f), f
