"""Design variables of the adjoint (minismac_gb300.design): CPU checks."""
import numpy as np

from minismac_gb300 import design, inputs


def test_hicks_henne_bump():
    x = np.linspace(0.0, 1.0, 2001)
    for i in range(1, 9):
        h = i / 9
        b = design.hicks_henne(x, h)
        assert b[0] == 0.0 and b[-1] == 0.0
        assert abs(x[np.argmax(b)] - h) < 1e-3       # peak at x = h
        assert abs(design.hicks_henne(np.array([h]), h)[0] - 1.0) < 1e-12
        assert np.all(b >= 0.0)
    assert np.all(design.hicks_henne(np.array([-0.5, 1.5]), 0.5) == 0.0)


def test_design_motion():
    g, rows = inputs.naca4_cgrid(79, 21)
    d = design.Design(g, rows)
    assert d.ndv == 17 and d.names[0] == "alpha"
    dx, dy, da = d.sensitivities()
    assert np.all(dx == 0.0) and da[0] == 1.0 and np.all(da[1:] == 0.0)
    dy3 = dy.reshape(d.ndv, g.kmax, g.jmax)
    assert np.all(dy3[0] == 0.0)
    # the far field and the wake cut do not move; the bumps move their own surface outward
    assert np.all(dy3[:, -1, :] == 0.0)
    wall = np.zeros(g.jmax, bool)
    wall[d.jwall] = True
    assert np.all(dy3[:, 0, ~wall] == 0.0)
    for r, n in enumerate(d.names[1:], start=1):
        side = n.split("_")[0]
        w = dy3[r, 0]
        if side == "upper":
            assert np.all(w[: d.jle + 1] == 0.0) and w.max() > 0.5 and w.min() >= 0.0
        else:
            assert np.all(w[d.jle:] == 0.0) and w.min() < -0.5 and w.max() <= 0.0
        # each k-line follows its wall point, fading to zero at the far field
        col = dy3[r, :, np.argmax(np.abs(w))]
        assert abs(col[0]) >= abs(col[-2]) >= 0.0
    # a moved grid is the base grid plus h times the motion
    gm, dal = d.moved("upper_3", 1e-3)
    np.testing.assert_allclose(gm.y - g.y, 1e-3 * dy3[3], rtol=0, atol=1e-15)
    assert dal == 0.0 and d.moved("alpha", 0.25)[1] == 0.25


def test_near_wall_cells_translate():
    """Near the wall the blending weight stays ~1 (cells move with the surface)."""
    g, rows = inputs.naca4_cgrid(119, 31)
    d = design.Design(g, rows)
    assert np.all(d.blend[0] == 1.0) and np.all(d.blend[-1] == 0.0)
    assert np.all(d.blend[1:4, d.jwall] > 0.999)
