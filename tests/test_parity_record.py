"""The committed record of the 5000-iteration comparison at 481x121 meets the parity bounds.

tests/golden/record_parity_481x121.py ran the plain FP64 GPU path and the oracle side by side
for 5000 iterations (line relaxation and LU-SGS) and wrote tests/golden/parity_481x121_5000.json.
This CPU test reads that record: the per-iteration L2 residual within 1e-10 relative over the
whole history, Cl and Cd within 1e-9, the final p, u, v within 1e-9 of the largest |q|.

The L-infinity residual resmax = max |s dj| (ref/step.f:613-756) is held to 1e-7 instead: it is
one near-wall point's residual scaled by dj ~ 1e8, a difference of nearly cancelling fluxes, so it
amplifies the rounding differences of the state (1e-10 in q after 5000 iterations) far more than
the L2 norm does.  Recorded with line relaxation: 2.6e-8 in resmax against 3.9e-12 in the L2
residual; LU-SGS is bit-identical.
"""
import json
import os

import pytest

RECORD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "parity_481x121_5000.json")


@pytest.mark.skipif(not os.path.exists(RECORD), reason="record not generated")
def test_long_parity_record_within_bounds():
    with open(RECORD) as fh:
        rec = json.load(fh)
    assert rec["iterations"] == 5000
    assert set(rec["schemes"]) == {"line relaxation", "LU-SGS"}
    for name, d in rec["schemes"].items():
        assert d["rhsnorm_rel"] < 1e-10, (name, d["rhsnorm_rel"])
        assert d["resmax_rel"] < 1e-7, (name, d["resmax_rel"])
        assert d["cl_rel"] < 1e-9 and d["cd_rel"] < 1e-9, name
        assert d["q_final_rel"] < 1e-9, name
        assert len(d["checkpoints"]) == 10
