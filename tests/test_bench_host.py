"""Host logic of the benchmark (CPU): the time-to-drop bookkeeping, the seeded batch workload
and the lookup of committed ncu traffic figures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class FakeSolver:
    """A solver whose residuals fall geometrically: rmax_n = 10^(-n / decade), the L2 norm
    r0 * 10^(-n / l2_decade), 2 ms of device time per iteration."""

    def __init__(self, decade, l2_decade, r0=3.0):
        self.n, self.decade, self.l2_decade, self.r0 = 0, decade, l2_decade, r0
        self.ms = 0.0

    def run(self, k):
        it = np.arange(self.n + 1, self.n + k + 1, dtype=np.float64)
        self.n += k
        self.ms = 2.0 * k
        return {"rmax": 10.0 ** (-it / self.decade), "rhsnorm": self.r0 * 10.0 ** (-(it - 1) / self.l2_decade),
                "cl": 0.3 + 1.0 / it, "cd": 0.1 + 1.0 / it}

    def last_run_ms(self):
        return self.ms


def test_converge_finds_the_first_iteration_of_each_target():
    s = FakeSolver(decade=100.0, l2_decade=50.0)
    r = bench.converge(s, target=1e-9, l2_drop=1e-10, max_iters=5000, chunk=300)
    # rmax <= 1e-9 first at n = 900; the L2 norm has dropped 1e-10 first at n = 501
    assert r["rmax_target"]["iterations"] == 900
    assert r["l2_drop_target"]["iterations"] == 501
    assert r["rmax_target"]["device_s"] == pytest.approx(900 * 2.0 / 1e3)
    assert r["l2_drop_target"]["device_s"] == pytest.approx(501 * 2.0 / 1e3)
    assert r["rmax_target"]["cl"] == pytest.approx(0.3 + 1.0 / 900)
    # it stops at the end of the chunk in which both targets are met
    assert r["iterations_run"] == 900 and r["ms_per_iter"] == pytest.approx(2.0)


def test_converge_reports_a_target_not_reached():
    s = FakeSolver(decade=1000.0, l2_decade=50.0)
    r = bench.converge(s, target=1e-9, l2_drop=1e-10, max_iters=2000, chunk=500)
    assert r["rmax_target"] is None and r["l2_drop_target"]["iterations"] == 501
    assert r["iterations_run"] == 2000
    assert r["rmax_last"] == pytest.approx(10.0 ** (-2000 / 1000.0))


def test_batch_cases_are_seeded_and_within_the_stated_ranges():
    a, b = bench.batch_cases(64), bench.batch_cases(64)
    assert a == b                      # the same seed gives the same cases
    assert bench.batch_cases(64, seed=1) != a
    for c in a:
        assert 0.0 <= c["m"] <= 0.06 and 0.2 <= c["p"] <= 0.6 and 0.08 <= c["t"] <= 0.18
        assert -4.0 <= c["alpha"] <= 12.0 and 5e5 <= c["reynum"] <= 5e6
        assert c["size"] in bench.BATCH_SIZES
    assert {c["size"] for c in a} == set(bench.BATCH_SIZES)  # 64 draws cover the four sizes


def test_ncu_traffic_lookup_matches_the_committed_summary():
    import json
    with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as fh:
        rec = json.load(fh)["kernels"][0]
    b, src = bench.ncu_traffic(rec["kernel"], rec["workload"])
    assert b == pytest.approx(rec["dram_bytes_per_launch"]) and src == rec.get("source")
    assert bench.ncu_traffic(rec["kernel"], "another workload") == (None, None)
