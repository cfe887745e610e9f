"""Design variables of the airfoil for the discrete adjoint.

The variables are the angle of attack (degrees) and Hicks-Henne sine bumps on the upper and
lower surfaces,

    b_i(x) = sin(pi * x ** (ln 0.5 / ln h_i)) ** 3,    h_i = i / (nbumps + 1),  i = 1..nbumps,

with x the chordwise position of a wall point (0 at the leading edge, 1 at the trailing edge;
b_i peaks at x = h_i and vanishes at both ends).  A bump of amplitude a moves the wall points of
its surface outward (upper: +y, lower: -y) by a * b_i(x), and the grid follows: the point k of a
wall point's k-line moves by the same amount times w = 1 - s_k / s_kmax, where s is the arc length
along that k-line from the wall.  Near the wall the cells translate with the surface; the far
field does not move.  The motion is linear in the amplitudes, so a grid at amplitudes a is
exactly x0 + sum_i a_i dx_i (the same map serves the adjoint's grid sensitivities and the
finite-difference checks).  The reference has no design variables; this parameterisation is part
of the differentiation form.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .inputs import Grid


def hicks_henne(x: np.ndarray, h: float, width: float = 3.0) -> np.ndarray:
    """sin(pi x^(ln 0.5 / ln h))^width on 0 <= x <= 1 (zero outside)."""
    x = np.asarray(x, dtype=np.float64)
    e = math.log(0.5) / math.log(h)
    xc = np.clip(x, 0.0, 1.0)
    b = np.sin(math.pi * xc ** e) ** width
    b[(x <= 0.0) | (x >= 1.0)] = 0.0
    return b


@dataclasses.dataclass
class Design:
    """Angle of attack plus ``nbumps`` bumps per surface on a C-grid whose wall is the k = 1 line
    of the bcmain.dat rows with ibcval 0 (lower surface before the leading edge, as in the
    reference's grids)."""

    grid: Grid
    bc_rows: list
    nbumps: int = 8

    def __post_init__(self):
        g = self.grid
        walls = [r for r in self.bc_rows if r.ibcval == 0 and r.kbeg == 1 and r.kend == 1]
        if len(walls) != 1:
            raise ValueError("expected one k = 1 wall")
        w = walls[0]
        jb = w.jbeg - 1
        je = (g.jmax if w.jend == -1 else g.jmax - 1 if w.jend == -2 else w.jend) - 1
        xw = g.x[0, jb:je + 1]
        jle = jb + int(np.argmin(xw))
        xle, xte = float(g.x[0, jle]), float(xw.max())
        self.jwall = np.arange(jb, je + 1)
        self.jle = jle
        self.xc = (g.x[0, jb:je + 1] - xle) / (xte - xle)
        # blending along each k-line: 1 at the wall, 0 at the far field
        seg = np.hypot(np.diff(g.x, axis=0), np.diff(g.y, axis=0))     # (kmax-1, jmax)
        s = np.vstack([np.zeros((1, g.jmax)), np.cumsum(seg, axis=0)])  # (kmax, jmax)
        self.blend = 1.0 - s / s[-1:, :]
        self.names = (["alpha"] + [f"upper_{i}" for i in range(1, self.nbumps + 1)]
                      + [f"lower_{i}" for i in range(1, self.nbumps + 1)])

    @property
    def ndv(self) -> int:
        return len(self.names)

    def motion(self, name: str):
        """(dx, dy, dalpha) of one variable: grid motion per unit (kmax x jmax arrays) and the
        change of alpha in degrees per unit."""
        g = self.grid
        dx = np.zeros((g.kmax, g.jmax))
        dy = np.zeros((g.kmax, g.jmax))
        if name == "alpha":
            return dx, dy, 1.0
        side, i = name.split("_")
        i = int(i)
        b = hicks_henne(self.xc, i / (self.nbumps + 1))
        upper = self.jwall > self.jle
        lower = self.jwall < self.jle
        mask = upper if side == "upper" else lower
        sgn = 1.0 if side == "upper" else -1.0
        for jj, bb, m in zip(self.jwall, b, mask):
            if m and bb != 0.0:
                dy[:, jj] = sgn * bb * self.blend[:, jj]
        return dx, dy, 0.0

    def sensitivities(self, names=None):
        """dxdb, dydb (ndv x N, j fastest) and dalpha (ndv) for the C ABI."""
        names = self.names if names is None else list(names)
        N = self.grid.jmax * self.grid.kmax
        dxdb = np.zeros((len(names), N))
        dydb = np.zeros((len(names), N))
        da = np.zeros(len(names))
        for r, n in enumerate(names):
            dx, dy, a = self.motion(n)
            dxdb[r], dydb[r], da[r] = dx.ravel(), dy.ravel(), a
        return dxdb, dydb, da

    def moved(self, name: str, h: float):
        """The grid and the alpha change at value h of one variable (all others at 0)."""
        dx, dy, a = self.motion(name)
        g = self.grid
        return Grid(g.jmax, g.kmax, g.x + h * dx, g.y + h * dy), h * a
