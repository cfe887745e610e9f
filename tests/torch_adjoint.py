"""torch.autograd.Function over the GPU solver and its discrete adjoint (test harness only).

``AirfoilCoefficients.apply(b, case)`` returns the tensor [Cl, Cd] of the converged flow for the
design-variable vector b (b[0]: change of alpha in degrees, then the Hicks-Henne amplitudes of
``design.Design``); its backward pass returns the adjoint gradients (smac_adjoint_*), so torch
optimisers and losses can drive the airfoil shape."""
import numpy as np
import torch

from minismac_gb300 import abi, adjoint, design


class Case:
    """A converged base flow and a factory of solvers for moved grids (warm-started from it)."""

    def __init__(self, params, grid, rows, make_solver):
        self.p, self.grid, self.rows, self.make = params, grid, rows, make_solver
        self.design = design.Design(grid, rows)
        base = make_solver(grid, 0.0)
        adjoint.converge(base)
        self.q0, self.c0 = base.get("q"), base.get_clift()
        base.close()

    def evaluate(self, b):
        b = np.asarray(b, dtype=np.float64)
        dxdb, dydb, da = self.design.sensitivities()
        g = self.grid
        x = g.x + (b @ dxdb).reshape(g.kmax, g.jmax)
        y = g.y + (b @ dydb).reshape(g.kmax, g.jmax)
        s = self.make(type(g)(g.jmax, g.kmax, x, y), float(b @ da))
        s.set_state(q=self.q0)
        s.set_clift(self.c0)
        c = adjoint.converge(s)
        r = adjoint.gradients(s, self.design)
        s.close()
        return c["cl"], c["cd"], r["cl"], r["cd"]


class AirfoilCoefficients(torch.autograd.Function):
    @staticmethod
    def forward(ctx, b, case):
        cl, cd, gcl, gcd = case.evaluate(b.detach().cpu().numpy())
        ctx.save_for_backward(torch.as_tensor(gcl, dtype=b.dtype), torch.as_tensor(gcd, dtype=b.dtype))
        return torch.tensor([cl, cd], dtype=b.dtype)

    @staticmethod
    def backward(ctx, gout):
        gcl, gcd = ctx.saved_tensors
        return gout[0] * gcl + gout[1] * gcd, None
