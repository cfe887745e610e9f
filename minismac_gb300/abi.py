"""ctypes mirror of include/smac_gb300.h (structs and constants).

Kept in one place so that the product wrapper (``minismac_gb300.solver``) and the test
harness agree on the struct layouts.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

MAX_BC = 64

OK, ERR_ARG, ERR_BC, ERR_NONFINITE, ERR_CUDA, ERR_UNSUPPORTED, ERR_NOMEM, ERR_TIMEOUT = range(8)
PREC_FP64, PREC_MIXED = 0, 1
ORDER_REFERENCE, ORDER_MULTICOLOR = 0, 1
WALLDIST_REFERENCE, WALLDIST_FIXED = 0, 1
LINES_PARTITIONED, LINES_SEQUENTIAL = 0, 1
BATCH_GRAPH, BATCH_PACKED_LINES, BATCH_QUEUE_LINES = 0, 1, 2

FIELD_Q, FIELD_ANUT, FIELD_VNUT, FIELD_S, FIELD_DQ, FIELD_RTXY, FIELD_DJ = range(7)
FIELD_BTC, FIELD_BJM, FIELD_BJP, FIELD_BKM, FIELD_BKP, FIELD_SMIN = range(7, 13)
FIELD_NCOMP = {FIELD_Q: 3, FIELD_ANUT: 1, FIELD_VNUT: 1, FIELD_S: 3, FIELD_DQ: 3, FIELD_RTXY: 6,
               FIELD_DJ: 1, FIELD_BTC: 9, FIELD_BJM: 9, FIELD_BJP: 9, FIELD_BKM: 9, FIELD_BKP: 9,
               FIELD_SMIN: 1}
FIELD_NAMES = {"q": FIELD_Q, "anut": FIELD_ANUT, "vnut": FIELD_VNUT, "s": FIELD_S, "dq": FIELD_DQ,
               "rtxy": FIELD_RTXY, "dj": FIELD_DJ, "btc": FIELD_BTC, "bjm": FIELD_BJM, "bjp": FIELD_BJP,
               "bkm": FIELD_BKM, "bkp": FIELD_BKP, "smin": FIELD_SMIN}


OBJ_CL, OBJ_CD = 0, 1
ADJ_FIELDS = {"lambda_cl": 0, "lambda_cd": 1, "dcl_dq": 2, "dcd_dq": 3, "df_dclift": 4, "jacobian": 5}


class SmacParams(C.Structure):
    _fields_ = [
        ("alpha", C.c_double), ("beta", C.c_double), ("dt", C.c_double), ("dtau", C.c_double),
        ("reynum", C.c_double), ("underr", C.c_double), ("pin", C.c_double), ("pout", C.c_double),
        ("cdis", C.c_double), ("anut_inf", C.c_double),
        ("impsch", C.c_int), ("ivis", C.c_int), ("iturb", C.c_int), ("njsp", C.c_int), ("nksp", C.c_int),
        ("ntjsp", C.c_int), ("ntksp", C.c_int), ("nbcimp", C.c_int), ("iflxo", C.c_int), ("itrans", C.c_int),
        ("wall_distance", C.c_int), ("precision", C.c_int), ("order", C.c_int), ("line_solver", C.c_int),
        ("visc_fp64", C.c_int), ("reserved", C.c_int * 2),
    ]


class SmacBCSpec(C.Structure):
    _fields_ = [("nbc", C.c_int)] + [(n, C.c_int * MAX_BC) for n in
                                     ("ibcval", "nzbc", "jbcb", "jbce", "kbcb", "kbce")]


class SmacIterOut(C.Structure):
    _fields_ = [
        ("nt", C.c_int), ("jres", C.c_int), ("kres", C.c_int), ("neq_res", C.c_int),
        ("resmax", C.c_double), ("resmax0", C.c_double), ("rmax", C.c_double), ("divmax", C.c_double),
        ("turres", C.c_double), ("rhsnorm", C.c_double), ("cd", C.c_double), ("cl", C.c_double),
        ("cm", C.c_double), ("cdp", C.c_double), ("clp", C.c_double),
    ]


HIST_FIELDS = ["nt", "jres", "kres", "neq_res", "resmax", "resmax0", "rmax", "divmax", "turres",
               "rhsnorm", "cd", "cl", "cm", "cdp", "clp"]


def hist_to_dict(arr) -> dict:
    return {f: np.array([getattr(h, f) for h in arr]) for f in HIST_FIELDS}


def default_params(**kw) -> SmacParams:
    """Reference defaults: hard-coded values of ref/initia.f (nbcimp, pin, pout) and
    inizone (njsp = nksp = 2, ntjsp = 2, ntksp = 0, iflxo = 3, cdis = 1, itrans = 0), and the
    flow values of the shipped ref/smac2d.in (overridable by keyword)."""
    p = SmacParams()
    p.alpha, p.beta, p.dt, p.dtau, p.reynum, p.underr = 10.0, 5.0, 1.0e12, 0.1, 1.5e6, 0.01
    p.pin, p.pout, p.cdis, p.anut_inf = 1.5, 1.0, 1.0, 0.0
    p.impsch, p.ivis, p.iturb = 1, 1, 1
    p.njsp, p.nksp, p.ntjsp, p.ntksp, p.nbcimp = 2, 2, 2, 0, 1
    p.iflxo, p.itrans = 3, 0
    p.wall_distance, p.precision, p.order = WALLDIST_REFERENCE, PREC_FP64, ORDER_REFERENCE
    p.line_solver = LINES_PARTITIONED
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def params_from_namelist(nl: dict, **kw) -> SmacParams:
    p = default_params()
    for key in ("alpha", "beta", "dt", "dtau", "reynum", "underr"):
        if key in nl:
            setattr(p, key, float(nl[key]))
    for key in ("impsch", "ivis", "iturb"):
        if key in nl:
            setattr(p, key, int(nl[key]))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def bcspec_from_rows(rows) -> SmacBCSpec:
    if not 0 < len(rows) <= MAX_BC:
        raise ValueError("between 1 and 64 BC rows are supported")
    b = SmacBCSpec()
    b.nbc = len(rows)
    for i, r in enumerate(rows):
        b.ibcval[i], b.nzbc[i], b.jbcb[i], b.jbce[i], b.kbcb[i], b.kbce[i] = (
            r.ibcval, r.zone, r.jbeg, r.jend, r.kbeg, r.kend)
    return b


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))
