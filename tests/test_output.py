"""The reference's output formats (XX line, Q2D.p3d, YAML summary): CPU checks."""
import datetime as dt

import numpy as np
import pytest

from minismac_gb300 import output


@pytest.mark.parametrize("v,w,d,scale,expect", [
    (1.2345e-3, 11, 3, 1, "  1.234E-03"),
    (0.0, 11, 3, 1, "  0.000E+00"),
    (-2.5e120, 12, 4, 1, " -2.5000+120"),
    (1.0, 12, 4, 1, "  1.0000E+00"),
    (1.5e6, 12, 4, 0, "  0.1500E+07"),
    (-0.012345678, 14, 6, 0, " -0.123457E-01"),
    (9.99996, 12, 4, 0, "  0.1000E+02"),
    (1e300, 8, 3, 1, "********"),
])
def test_fortran_e(v, w, d, scale, expect):
    assert output.fortran_e(v, w, d, scale) == expect


@pytest.mark.parametrize("v,w,d,scale,expect", [
    (0.0, 5, 2, 1, " 0.00"),
    (-0.1234567, 10, 6, 0, " -0.123457"),
    (3.0, 10, 6, 0, "  3.000000"),
    (1234.5, 10, 6, 0, "**********"),
    (0.5, 4, 3, 0, ".500"),
])
def test_fortran_f(v, w, d, scale, expect):
    assert output.fortran_f(v, w, d, scale) == expect


def test_xx_line_layout():
    s = output.xx_line(7, 1.0, 0.5, 2e-5, 10, 1, 1, 0.123, 0.0123, 1.1)
    # 'XX' + i5 + 3 x e11.3 + 3 x i6 + 3 x e12.4
    assert len(s) == 2 + 5 + 33 + 18 + 36
    assert s.startswith("XX    7  1.000E+00")
    assert s[40:58] == "    10     1     1"
    assert output.xx_header_due(1) and output.xx_header_due(26) and not output.xx_header_due(25)


def test_q2d_round_trip(tmp_path):
    jmax, kmax = 7, 5
    rng = np.random.default_rng(3)
    q = rng.uniform(-1.0, 1.0, size=3 * jmax * kmax)
    f = tmp_path / "Q2D.p3d"
    output.write_q2d(str(f), q, jmax, kmax, alpha=10.0, reynum=1.5e6, cputime=12.5)
    lines = f.read_text().splitlines()
    assert lines[0] == "           1" and lines[1] == "           7           5"
    assert lines[2] == " 0.00   1.00000E+01   1.50000E+06   1.25000E+01"
    assert all(len(ln) <= 60 for ln in lines[3:])
    j, k, head, v = output.read_q2d(str(f))
    assert (j, k) == (jmax, kmax) and head == [0.0, 10.0, 1.5e6, 12.5]
    ref = output.q2d_variables(q, jmax, kmax)
    np.testing.assert_allclose(v, ref, atol=5e-7, rtol=0)
    # fourth variable: p / 0.4 with the reference's REAL*4 literal
    qq = q.reshape(3, kmax, jmax)
    np.testing.assert_array_equal(ref[3], qq[0] / np.float64(np.float32(0.4)) + 0.5 * (qq[1] ** 2 + qq[2] ** 2))


def test_yaml_summary_keys_in_reference_order():
    when = dt.datetime(2026, 1, 2, 3, 4, 5)
    name = output.yaml_filename("NACA 4412 Airfoil", 119, 31, 200, host="box", when=when)
    assert name == "smac2d_NACA_4412_Airfoil_box_119x31_1ranks_0threads_200iters_double_2026_01_02_03_04_05.yaml"
    text = output.yaml_summary(title="SMAC2D", geometry="NACA 4412 Airfoil", grid_file="xy.dat", jmax=119, kmax=31,
                               beta=5.0, dtau=0.1, reynum=1.5e6, alpha=10.0, impsch=1, cd=np.float64(0.02),
                               cl=1.1, cm=-0.1, rmax=0.3, ntmax=200, init_sec=1.0, solve_sec=2.0, filename=name,
                               host="box", when=when)
    keys = [ln.split(":")[0].strip() for ln in text.splitlines()]
    expect = ["user", "code", "host", "title", "geometry", "date_yyyy_mm_dd", "time_of_day", "num_grids",
              "mpi_ranks", "num_threads_per_node", "total_processes", "grid_file", "largest_dim", "j-dim",
              "k-dim", "total_points", "beta", "fp_precision", "dtau", "reynolds_number",
              "angle_of_attack_degs", "implicit_scheme", "airfoil", "cd", "cl", "cm", "residual",
              "sec_per_iteration", "microsec_per_iter_per_point", "number_of_iterations", "alpha_deg",
              "initialize_sec", "send_subgrids_sec", "solve_sec", "total_time_sec", "yaml_filename"]
    assert keys == expect
    vals = dict(ln.split(":", 1) for ln in text.splitlines())
    assert float(vals["   cd"]) == 0.02
    assert float(vals["microsec_per_iter_per_point"]) == pytest.approx(2.0 / 200 / (119 * 31) * 1e6, rel=1e-4)
    assert vals["implicit_scheme"].strip() == "line relaxation"
