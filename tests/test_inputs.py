"""Input formats (smac2d.in, xy.dat, bcmain.dat) and the synthetic C-grid family."""
import os

import numpy as np
import pytest

from minismac_gb300 import abi, inputs

from golden_case import reference_inputs_dir

REF = reference_inputs_dir()


def test_namelist_parse():
    text = """ $input
  alpha=10.0d0   ! degs
  beta=5.0d0
  dt=1.0d12
  impsch=2
  geometry='NACA 4412 Airfoil'   ! name
  zz_run_default_input=.false.
  $end
"""
    nl = inputs.read_namelist(text)
    assert nl["alpha"] == 10.0 and nl["dt"] == 1e12 and nl["impsch"] == 2
    assert nl["geometry"] == "NACA 4412 Airfoil" and nl["zz_run_default_input"] is False
    p = abi.params_from_namelist(nl)
    assert p.alpha == 10.0 and p.impsch == 2 and p.njsp == 2 and p.ntksp == 0


def test_bcmain_roundtrip(tmp_path):
    rows = inputs.cgrid_bc_rows(119, 20)
    f = tmp_path / "bcmain.dat"
    inputs.write_bcmain(str(f), rows, "test")
    back = inputs.read_bcmain(str(f))
    assert back == rows
    assert [r.ibcval for r in rows] == [31, 31, 0, 25, 60, 60]


def test_xy_roundtrip(tmp_path):
    g, _ = inputs.naca4_cgrid(59, 17)
    f = tmp_path / "xy.dat"
    inputs.write_xy(str(f), g)
    h = inputs.read_xy(str(f))
    assert (h.jmax, h.kmax) == (59, 17)
    assert np.array_equal(h.x, g.x) and np.array_equal(h.y, g.y)


@pytest.mark.parametrize("jk", [(119, 31), (241, 61), (481, 121)])
def test_cgrid_geometry(jk):
    jmax, kmax = jk
    g, rows = inputs.naca4_cgrid(jmax, kmax)
    x, y = g.x, g.y
    nw = inputs.wake_points(jmax)
    # wake points coincide pairwise across the cut (j <-> jmax+1-j on k = 1)
    assert np.array_equal(x[0, :nw], x[0, ::-1][:nw]) and np.array_equal(y[0, :nw], y[0, ::-1][:nw])
    # first normal spacing and far field
    d1 = np.hypot(x[1] - x[0], y[1] - y[0])
    assert abs(d1.min() - 1e-5) < 1e-7
    assert np.hypot(x[-1] - 1.0, y[-1]).min() > 9.9
    # positive Jacobian everywhere (same central / one-sided differences as the metric)
    xj, yj = np.gradient(x, axis=1), np.gradient(y, axis=1)
    xk, yk = np.gradient(x, axis=0), np.gradient(y, axis=0)
    assert ((xj * yk - xk * yj) > 0).all()
    # leading edge at the middle index
    assert abs(x[0, (jmax - 1) // 2]) < 1e-12


@pytest.mark.skipif(REF is None, reason="SMAC_REFERENCE_DIR unset or without the reference's ref/ inputs")
def test_reference_inputs_parse():
    g = inputs.read_xy(os.path.join(REF, "xy.dat_original_119x31"))
    rows = inputs.read_bcmain(os.path.join(REF, "bcmain.dat_original_119x31"))
    assert (g.jmax, g.kmax) == (119, 31)
    assert rows == inputs.cgrid_bc_rows(119, 20)
