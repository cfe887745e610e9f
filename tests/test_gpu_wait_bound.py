"""The bounded device waits of the reference-order line sweeps.

The partitioned line sweep waits, at the start of every line, for the bulk copy of its operator
block into shared memory.  Every such wait gives up after about a second, records
SMAC_ERR_TIMEOUT in the iteration's device status and lets the kernel finish its lines without
waiting, so that no CTA is left behind a cluster barrier and no copy stays in flight.  Here the
wait is made to run out on purpose, on the host's request and without any fault: with
SMAC_TEST_STALL_WAIT set when the context is created, the first line of the next smac_step's
first sweep also waits on a barrier that nothing completes.  The step must come back with
SMAC_ERR_TIMEOUT, and the context must stay usable: after the state is put back, further steps
give exactly the results of a fresh context.
"""
import numpy as np
import pytest

from minismac_gb300 import abi, inputs

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_reports_timeout_and_context_recovers(cuda_lib, monkeypatch):
    from minismac_gb300.solver import SmacError, Solver
    g, rows = inputs.naca4_cgrid(119, 31)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6)
    fresh = Solver(p, g, rows)
    q0, a0 = fresh.get("q"), fresh.get("anut")
    monkeypatch.setenv("SMAC_TEST_STALL_WAIT", "1")
    s = Solver(p, g, rows)
    monkeypatch.delenv("SMAC_TEST_STALL_WAIT")
    with pytest.raises(SmacError) as err:
        s.step()
    assert f"({abi.ERR_TIMEOUT})" in str(err.value) and "ran out of time" in str(err.value)
    # the context is still usable: restore the initial state and compare with a fresh context
    s.set_state(q0, a0)
    s.set_clift(0.0)
    for _ in range(3):
        o_s, o_f = s.step(), fresh.step()
        assert o_s.cl == o_f.cl and o_s.rhsnorm == o_f.rhsnorm
    np.testing.assert_array_equal(s.get("q"), fresh.get("q"))
    s.close()
    fresh.close()


def test_batch_queue_wait_that_runs_out_reports_timeout(cuda_lib, monkeypatch):
    """The persistent line-sweep launch of a batch: every item waits (bounded) for the previous
    phase of its case.  With SMAC_TEST_STALL_WAIT set when the batch is created, the first
    item of the next run also waits for one item more than its phase will ever count; that wait
    gives up after about a second, the launch finishes without waiting any more, and the run
    returns SMAC_ERR_TIMEOUT.  Afterwards, with the cases' states put back, the batch gives the
    mean flow and forces of a fresh batch again."""
    from minismac_gb300.solver import Batch, SmacError, Solver

    def make():
        out = []
        for (jm, km), a in (((119, 31), 2.0), ((79, 21), 6.0)):
            g, rows = inputs.naca4_cgrid(jm, km)
            p = abi.default_params(alpha=a, beta=10.0, reynum=1e6, order=abi.ORDER_MULTICOLOR,
                                   precision=abi.PREC_MIXED, wall_distance=abi.WALLDIST_FIXED)
            out.append(Solver(p, g, rows))
        return out

    monkeypatch.setenv("SMAC_ZEBRA_SHAPE", "-4,-4")
    fresh_cases = make()
    start = [(s.get("q"), s.get("anut")) for s in fresh_cases]
    fresh = Batch(fresh_cases, queue=True, warps_per_line=4)
    cases = make()
    monkeypatch.setenv("SMAC_TEST_STALL_WAIT", "1")
    b = Batch(cases, queue=True, warps_per_line=4)
    monkeypatch.delenv("SMAC_TEST_STALL_WAIT")
    with pytest.raises(SmacError) as err:
        b.run(2)
    assert f"({abi.ERR_TIMEOUT})" in str(err.value) and "ran out of time" in str(err.value)
    for s, (q0, a0) in zip(cases, start):
        s.set_state(q0, a0)
        s.set_clift(0.0)
    hb, hf = b.run(3), fresh.run(3)
    for i, s in enumerate(cases):
        for key in ("rhsnorm", "cl", "cd"):
            np.testing.assert_array_equal(hb[i][key], hf[i][key], err_msg=f"case {i} {key}")
        np.testing.assert_array_equal(s.get("q"), fresh_cases[i].get("q"))
    b.close()
    fresh.close()
