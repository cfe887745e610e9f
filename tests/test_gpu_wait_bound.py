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
