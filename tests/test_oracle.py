"""CPU checks of the oracle itself: the golden fixtures of the reference's shipped 119x31 case
and the self-consistency properties of the discretisation (no GPU needed)."""
import os
import platform

import numpy as np
import pytest

from minismac_gb300 import abi, inputs
from oracle.oracle_py import Oracle

from golden_case import MEAN_FLOW_KEYS, load_golden, reference_inputs_dir

@pytest.mark.parametrize("impsch", [1, 2])
def test_golden_history_reproduced(impsch):
    """The oracle rerun on the shipped grid, BCs and namelist reproduces the committed history
    and final fields (bit for bit on the machine that wrote them)."""
    z, grid, rows, p = load_golden(impsch)
    n = z["hist_rmax"].size
    o = Oracle(p, grid, rows)
    h = o.run(n)
    exact = platform.machine() in ("x86_64", "AMD64")
    for k in MEAN_FLOW_KEYS:
        ref = z[f"hist_{k}"]
        if exact:
            np.testing.assert_array_equal(h[k], ref, err_msg=k)
        else:  # another libm: the mean flow uses no transcendental beyond cos/sin of alpha
            np.testing.assert_allclose(h[k], ref, rtol=1e-12, atol=1e-14, err_msg=k)
    q = o.get("q")
    if exact:
        np.testing.assert_array_equal(q, z["q"])
        np.testing.assert_array_equal(o.get("anut"), z["anut"])
        np.testing.assert_array_equal(h["turres"], z["hist_turres"])
    else:
        np.testing.assert_allclose(q, z["q"], rtol=0, atol=1e-12)


@pytest.mark.skipif(reference_inputs_dir() is None,
                    reason="SMAC_REFERENCE_DIR unset or without the reference's ref/ inputs")
def test_golden_inputs_are_the_shipped_files():
    REF_INPUTS = reference_inputs_dir()
    z, grid, rows, p = load_golden(1)
    g = inputs.read_xy(os.path.join(REF_INPUTS, "xy.dat_original_119x31"))
    x, y = g.flat()
    np.testing.assert_array_equal(x, z["x"])
    np.testing.assert_array_equal(y, z["y"])
    r = inputs.read_bcmain(os.path.join(REF_INPUTS, "bcmain.dat_original_119x31"))
    assert [(b.ibcval, b.zone, b.jbeg, b.jend, b.kbeg, b.kend) for b in r] == [tuple(b) for b in z["bc"].tolist()]
    nl = inputs.read_namelist(os.path.join(REF_INPUTS, "smac2d.in"))
    for k in ("alpha", "beta", "dt", "dtau", "reynum", "underr"):
        assert getattr(p, k) == float(nl[k])


def test_golden_shipped_run_is_sane():
    z, *_ = load_golden(1)
    assert np.all(np.isfinite(z["q"])) and np.all(np.isfinite(z["hist_rhsnorm"]))
    assert z["hist_rmax"][0] == 1.0 or z["hist_rmax"][0] > 0
    # the far-field vortex uses the lift of the previous iteration: Cl of the 10-degree case
    # settles near 1.1 within the 200 iterations of the shipped namelist
    assert 0.8 < z["hist_cl"][-1] < 1.5


@pytest.mark.parametrize("ivis", [0, 1])
def test_freestream_preservation(ivis):
    """A uniform flow gives a zero residual at every interior point of a curvilinear grid:
    the face metrics of the flux and viscous terms telescope exactly."""
    g, rows = inputs.naca4_cgrid(119, 31)
    p = abi.default_params(alpha=5.0, ivis=ivis, iturb=0)
    o = Oracle(p, g, rows)
    a = np.deg2rad(5.0)
    q = o.get("q").reshape(3, 31, 119)
    q[0], q[1], q[2] = 1.0, np.cos(a), np.sin(a)
    o.set("q", q.ravel())
    o.stage_assemble()
    s = o.get("s").reshape(3, 31, 119)
    assert np.abs(s[:, 1:-1, 1:-1]).max() < 1e-13


def test_symmetric_airfoil_gives_mirror_symmetric_residual():
    """NACA 0012 at zero incidence on a mirror-symmetric C-grid: the assembled residual of the
    initial state is mirror symmetric across the wake cut (p, u even; v odd)."""
    jm, km = 119, 31
    g, rows = inputs.naca4_cgrid(jm, km, m=0.0, p=0.4, t=0.12)
    assert np.abs(g.x - g.x[:, ::-1]).max() < 1e-12 and np.abs(g.y + g.y[:, ::-1]).max() < 1e-12
    p = abi.default_params(alpha=0.0, beta=10.0, reynum=1000.0)
    o = Oracle(p, g, rows)
    o.stage_assemble()
    s = o.get("s").reshape(3, km, jm)
    scale = np.abs(s).max()
    assert np.abs(s[0] - s[0][:, ::-1]).max() < 1e-13 * scale
    assert np.abs(s[1] - s[1][:, ::-1]).max() < 1e-13 * scale
    assert np.abs(s[2] + s[2][:, ::-1]).max() < 1e-13 * scale


def test_lr_and_lusgs_share_the_residual():
    """Line relaxation and LU-SGS solve for the same fixed point: on the same state (here the
    one 50 line-relaxation iterations reach) both schemes assemble the same residual."""
    g, rows = inputs.naca4_cgrid(79, 21)

    def params(imp):
        return abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0, impsch=imp)

    lr = Oracle(params(1), g, rows)
    lr.run(50)
    state = lr.get("q")
    res = []
    for imp in (1, 2):
        o = Oracle(params(imp), g, rows)
        o.set("q", state)
        o.stage_assemble()
        res.append(o.get("s"))
    np.testing.assert_array_equal(res[0], res[1])


def test_residual_drops_on_a_converging_case():
    """Laminar Re = 1000 (the reference's mean flow is laminar): line relaxation with a large
    pseudo-time step drops the maximum residual by more than four decades in 1500 iterations."""
    g, rows = inputs.naca4_cgrid(59, 17)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0, impsch=1)
    h = Oracle(p, g, rows).run(1500)
    assert h["rmax"][-1] < 1e-4
    assert np.all(np.isfinite(h["cl"]))
