"""The reference-style host loop on the GPU: smac2d.in + xy.dat + bcmain.dat in, XX lines,
YAML summary and Q2D.p3d out, checked against the golden fixtures of the shipped case."""
import io
import os

import numpy as np
import pytest

from golden_case import load_golden
from minismac_gb300 import inputs, output

pytestmark = pytest.mark.gpu

NAMELIST = """ $input
  alpha=10.0d0
  beta=5.0d0
  dt=1.0d12
  dtau=0.1d0
  geometry='NACA 4412 Airfoil'
  impsch=1
  iturb=1
  ivis=1
  ntmax={ntmax}
  reynum=1.5d6
  title='SMAC2D -- Sandia MiniAero Code 2D'
  underr=0.01d0
  write_plot3d_q_file=.true.
  bcmain_directory='{d}'
  bcmain_filename='bcmain.dat'
  xygrid_directory='{d}'
  xygrid_filename='xy.dat'
  $end
"""


def test_driver_reproduces_shipped_history(cuda_lib, tmp_path):
    from minismac_gb300 import driver
    z, grid, rows, p = load_golden(1)
    n = 30
    inputs.write_xy(str(tmp_path / "xy.dat"), grid)
    inputs.write_bcmain(str(tmp_path / "bcmain.dat"), rows, "shipped 119x31 case")
    (tmp_path / "smac2d.in").write_text(NAMELIST.format(ntmax=n, d=str(tmp_path)))
    buf = io.StringIO()
    res = driver.run([str(tmp_path / "smac2d.in"), "--outdir", str(tmp_path / "out"), "--line-solver", "1"],
                     stdout=buf)
    xx = [ln for ln in buf.getvalue().splitlines() if ln.startswith("XX")]
    assert len(xx) == n
    for i, ln in enumerate(xx):
        assert ln == output.xx_line(i + 1, z["hist_rmax"][i], z["hist_divmax"][i], float(ln[29:40]),
                                    z["hist_jres"][i], z["hist_kres"][i], 1, float(ln[58:70]),
                                    z["hist_cd"][i], z["hist_cl"][i])
    assert res["last"].cl == z["hist_cl"][n - 1]
    assert os.path.isfile(res["yaml"])
    j, k, head, v = output.read_q2d(str(tmp_path / "out" / "Q2D.p3d"))
    assert (j, k) == (grid.jmax, grid.kmax) and head[1] == 10.0
    assert np.all(np.isfinite(v)) and np.all(v[0] == 1.0)
