"""Host logic of the adjoint helpers (minismac_gb300.adjoint) with fake solvers: CPU only."""
import numpy as np

from minismac_gb300 import adjoint, design, inputs


class FakeSolver:
    """A 'solver' whose residual halves every iteration down to a floor and whose Cl and Cd are
    fixed functions of the grid and alpha (so central differences are known exactly)."""

    def __init__(self, grid=None, dalpha=0.0, floor=1e-9):
        self.grid, self.dalpha, self.floor = grid, dalpha, floor
        self.r, self.it, self.q, self.clift = 1.0, 0, None, None

    def coeffs(self):
        y = 0.0 if self.grid is None else float(np.sum(self.grid.y))
        return 0.3 + 0.1 * self.dalpha + 1e-3 * y, 0.05 + 0.02 * self.dalpha ** 2 - 2e-4 * y

    def run(self, n):
        res = []
        for _ in range(n):
            self.r = max(self.r * 0.5, self.floor)
            res.append(self.r)
            self.it += 1
        cl, cd = self.coeffs()
        return {"resmax": np.array(res), "cl": np.full(n, cl), "cd": np.full(n, cd)}

    def set_state(self, q=None, turvar=None):
        self.q = q

    def set_clift(self, c):
        self.clift = c

    def close(self):
        pass


def test_converge_stops_at_the_floor():
    s = FakeSolver(floor=1e-12)
    info = adjoint.converge(s, max_iter=100000, chunk=100)
    assert info["resmax"] == 1e-12
    # stops a few chunks after the floor is reached, far before max_iter
    assert info["iterations"] <= 500


def test_converge_respects_max_iter():
    class Slow(FakeSolver):
        def run(self, n):
            h = super().run(n)
            h["cl"] = h["cl"] + 1e-6 * self.it  # Cl keeps moving: never converged
            return h
    info = adjoint.converge(Slow(), max_iter=1000, chunk=100)
    assert info["iterations"] == 1000


def test_finite_differences_are_central_and_warm_started():
    g, rows = inputs.naca4_cgrid(39, 11)
    d = design.Design(g, rows, nbumps=2)
    made = []

    def make(grid, dalpha):
        s = FakeSolver(grid, dalpha)
        made.append(s)
        return s

    q0 = np.arange(5.0)
    h = 1e-3
    fd = adjoint.finite_differences(make, d, ["alpha", "upper_1"], h, q0, 0.42, chunk=50)
    # alpha: dCl/dalpha = 0.1 exactly, dCd/dalpha = 0 at 0 (central difference of a square)
    assert abs(fd["cl"][0] - 0.1) < 1e-12 and abs(fd["cd"][0]) < 1e-12
    # a bump: Cl, Cd linear in sum(y), the motion linear in the amplitude
    dy = d.motion("upper_1")[1].sum()
    assert abs(fd["cl"][1] - 1e-3 * dy) < 1e-9 and abs(fd["cd"][1] + 2e-4 * dy) < 1e-9
    assert len(made) == 4 and all(s.clift == 0.42 and s.q is q0 for s in made)


def test_gradients_call_sequence():
    g, rows = inputs.naca4_cgrid(39, 11)
    d = design.Design(g, rows, nbumps=2)
    calls = []

    class FakeAdj:
        def adjoint_prepare(self):
            calls.append("prepare")

        def adjoint_solve(self, obj, rtol, max_iter):
            calls.append(("solve", obj))
            return {"iterations": 3, "rel_resid": 1e-12}

        def adjoint_gradient(self, obj, dxdb, dydb, da):
            calls.append(("gradient", obj, dxdb.shape, dydb.shape, tuple(da)))
            return np.ones(len(da)) * (1.0 if obj == "cl" else 2.0)

    r = adjoint.gradients(FakeAdj(), d)
    assert calls[0] == "prepare"
    assert [c[1] for c in calls if c[0] == "solve"] == ["cl", "cd"]
    g_calls = [c for c in calls if c[0] == "gradient"]
    assert g_calls[0][2] == (d.ndv, g.jmax * g.kmax) and g_calls[0][4][0] == 1.0
    assert np.all(r["cl"] == 1.0) and np.all(r["cd"] == 2.0) and r["names"] == d.names
