"""Discrete adjoint on the GPU (smac_adjoint_*): the steady equations against the assembled
right-hand side, their exact Jacobian against central differences, the transposed product,
and the gradients of Cl and Cd against central finite differences of the converged solver.

The converging case is laminar Re = 1000 (the reference's mean flow is laminar; at its Re = 1e6
it has no steady state).  The finite-difference checks use the FP64 viscous fluxes
(visc_fp64 = 1): the reference's REAL*4 viscous scratch makes the residual a step function at
the 1e-7 level, which a difference quotient with step 1e-6 cannot see through."""
import numpy as np
import pytest

from minismac_gb300 import abi, adjoint, design, inputs

pytestmark = pytest.mark.gpu


def case(jm=79, km=21, visc64=1, **kw):
    g, rows = inputs.naca4_cgrid(jm, km)
    kw.setdefault("alpha", 5.0)
    p = abi.default_params(beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0, impsch=1, iturb=0,
                           visc_fp64=visc64, **kw)
    return g, rows, p


def wake_rows(rows, jmax, N):
    """Indices (into 3N) of the wake-cut rows and the (jt, jb) pairs, 0-based."""
    def idx(v):  # the reference's negative indices: -1 -> jmax, -2 -> jmax - 1 (1-based)
        return jmax + 1 + v if v < 0 else v

    a, b = [r for r in rows if r.ibcval == 60]
    pairs = []
    for s, t in ((a, b), (b, a)):
        for i, jt in enumerate(range(idx(s.jbeg) - 1, idx(s.jend))):
            pairs.append((jt, idx(t.jend) - 1 - i))
    idx = np.array([jt + N * n for jt, _ in pairs for n in range(3)])
    return idx, pairs


def test_steady_equations_are_the_assembled_rhs(cuda_lib):
    from minismac_gb300.solver import Solver
    for visc64 in (0, 1):
        g, rows, p = case(visc64=visc64)
        s = Solver(p, g, rows)
        s.run(40)
        F = s.adjoint_residual()
        s.stage_assemble()
        rhs = s.get("s")
        q = s.get("q")
        N = g.jmax * g.kmax
        widx, pairs = wake_rows(rows, g.jmax, N)
        keep = np.ones(3 * N, bool)
        keep[widx] = False
        np.testing.assert_array_equal(F[keep], rhs[keep])
        for jt, jb in pairs:
            for n in range(3):
                want = 0.5 * (q[jt + g.jmax + N * n] + q[jb + g.jmax + N * n]) - q[jt + N * n]
                assert F[jt + N * n] == want


def test_jacobian_matches_central_differences(cuda_lib):
    from minismac_gb300.solver import Solver
    g, rows, p = case()
    s = Solver(p, g, rows)
    s.run(300)
    q0 = s.get("q")
    c0 = s.get_clift()
    s.adjoint_prepare()
    N = g.jmax * g.kmax
    rng = np.random.default_rng(11)
    v = rng.standard_normal(3 * N)
    Av = s.adjoint_jacvec(v)
    fc = s.adjoint_get("df_dclift")
    gcl = s.adjoint_get("dcl_dq")
    Fq_v = Av - fc * (gcl @ v)
    h = 1e-6

    def F_at(q):
        s.set_state(q=q)
        s.set_clift(c0)
        return s.adjoint_residual()

    fd = (F_at(q0 + h * v) - F_at(q0 - h * v)) / (2 * h)
    # interior rows and each boundary edge against their own scale
    kk, jj = np.divmod(np.arange(N), g.jmax)
    regions = {"interior": (jj > 0) & (jj < g.jmax - 1) & (kk > 0) & (kk < g.kmax - 1),
               "wall/wake": kk == 0, "far field": kk == g.kmax - 1,
               "outflow": ((jj == 0) | (jj == g.jmax - 1)) & (kk > 0) & (kk < g.kmax - 1)}
    for name, m in regions.items():
        m3 = np.tile(m, 3)
        err = np.abs(fd[m3] - Fq_v[m3]).max()
        scale = np.abs(Fq_v[m3]).max()
        assert err <= 1e-6 * scale, (name, err, scale)
    # dF/dclift: only the far-field rows depend on the vortex
    s.set_state(q=q0)
    s.set_clift(c0 + h)
    Fp = s.adjoint_residual()
    s.set_clift(c0 - h)
    Fm = s.adjoint_residual()
    np.testing.assert_allclose((Fp - Fm) / (2 * h), fc, rtol=0, atol=1e-7 * np.abs(fc).max())
    # dCl/dq: Cl is linear in q
    cl = []
    for sg in (1.0, -1.0):
        s.set_state(q=q0 + sg * h * v)
        s.set_clift(c0)
        s.adjoint_prepare()
        cl.append(s.adjoint_forces()[0])
    assert abs((cl[0] - cl[1]) / (2 * h) - gcl @ v) <= 1e-6 * abs(gcl @ v)


def test_transposed_product(cuda_lib):
    from minismac_gb300.solver import Solver
    g, rows, p = case()
    s = Solver(p, g, rows)
    s.run(100)
    s.adjoint_prepare()
    N = g.jmax * g.kmax
    rng = np.random.default_rng(5)
    for _ in range(3):
        v, w = rng.standard_normal(3 * N), rng.standard_normal(3 * N)
        a = w @ s.adjoint_jacvec(v)
        b = s.adjoint_jacvec(w, transpose=True) @ v
        assert abs(a - b) <= 1e-13 * np.linalg.norm(w) * np.linalg.norm(s.adjoint_jacvec(v))


def make_factory(p, rows, precision=abi.PREC_MIXED, order=abi.ORDER_MULTICOLOR):
    from minismac_gb300.solver import Solver

    def make(grid, dalpha):
        q = abi.SmacParams.from_buffer_copy(p)
        q.alpha = p.alpha + dalpha
        q.precision, q.order = precision, order
        return Solver(q, grid, rows)
    return make


@pytest.fixture(scope="module")
def converged_79():
    from minismac_gb300.solver import Solver
    g, rows, p = case()
    make = make_factory(p, rows)
    s = make(g, 0.0)
    info = adjoint.converge(s)
    return g, rows, p, s, info, make


def test_adjoint_gradients_match_finite_differences(cuda_lib, converged_79):
    g, rows, p, s, info, make = converged_79
    # converged to the round-off floor: Cl stopped moving (resmax, scaled by the near-wall
    # Jacobian ~1e8, bottoms out near 1e-9)
    assert info["iterations"] < 60000 and info["resmax"] < 1e-8, info
    d = design.Design(g, rows)
    res = adjoint.gradients(s, d)
    for obj in ("cl", "cd"):
        assert res["stats"][obj]["rel_resid"] < 1e-10, res["stats"]
    names = ["alpha", "upper_2", "lower_4", "upper_7"]
    q0 = s.get("q")
    fd = adjoint.finite_differences(make, d, names, 1e-6, q0, s.get_clift())
    for obj in ("cl", "cd"):
        ad = np.array([res[obj][d.names.index(n)] for n in names])
        print(obj, "adjoint", ad, "fd", fd[obj], "stats", res["stats"][obj], "fd its", fd["iterations"])
        err = np.abs(ad - fd[obj])
        scale = np.maximum(np.abs(fd[obj]), 1e-3 * np.abs(fd[obj]).max())
        assert np.all(err <= 1e-6 * scale + 1e-10), (obj, ad, fd[obj], err / scale)


def _oracle_converged(args):
    """One oracle solve on a moved grid from a warm start, to its round-off floor (runs in a
    spawned process)."""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from minismac_gb300 import abi as _abi
    from minismac_gb300 import adjoint as _adjoint
    from oracle.oracle_py import Oracle
    params_bytes, grid, rows, q0, clift0 = args
    p = _abi.SmacParams.from_buffer_copy(params_bytes)
    o = Oracle(p, grid, rows)
    o.set("q", q0)
    o.set_clift(clift0)
    c = _adjoint.converge(o, max_iter=60000, chunk=1000)
    o.close()
    return c


def test_adjoint_gradients_match_reference_finite_differences(cuda_lib, converged_79):
    """The same gradients against central differences of the oracle (the reference's algorithm
    on the CPU): alpha and one lower-surface bump, four oracle solves in parallel processes."""
    import multiprocessing as mp
    from oracle.oracle_py import build as build_oracle
    build_oracle()
    g, rows, p, s, info, make = converged_79
    d = design.Design(g, rows)
    names = ["alpha", "lower_4"]
    res = adjoint.gradients(s, d, names=names)
    q0, c0 = s.get("q"), s.get_clift()
    h = 1e-6
    jobs = []
    for n in names:
        for sg in (1.0, -1.0):
            grid, da = d.moved(n, sg * h)
            q = abi.SmacParams.from_buffer_copy(p)
            q.alpha = p.alpha + da
            jobs.append((bytes(q), grid, rows, q0, c0))
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        out = pool.map(_oracle_converged, jobs)
    for i, n in enumerate(names):
        for obj in ("cl", "cd"):
            fd = (out[2 * i][obj] - out[2 * i + 1][obj]) / (2 * h)
            ad = res[obj][i]
            print(n, obj, "adjoint", ad, "oracle fd", fd, "oracle its", out[2 * i]["iterations"])
            assert abs(ad - fd) <= 1e-6 * abs(fd) + 1e-10, (n, obj, ad, fd)


def test_torch_autograd_function(cuda_lib):
    """torch drives the adjoint: d(Cl - 3 Cd)/db by backward() at a moved design point equals the
    adjoint gradients, and its alpha entry a central difference of the forward pass."""
    torch = pytest.importorskip("torch")
    from torch_adjoint import AirfoilCoefficients, Case
    g, rows, p = case()
    case_ = Case(p, g, rows, make_factory(p, rows))
    b0 = np.zeros(case_.design.ndv)
    b0[0], b0[3], b0[12] = 0.5, 2e-3, -1e-3
    b = torch.tensor(b0, requires_grad=True)
    y = AirfoilCoefficients.apply(b, case_)
    loss = y[0] - 3.0 * y[1]
    loss.backward()
    h = 1e-6
    e = np.zeros_like(b0)
    e[0] = h
    yp = AirfoilCoefficients.apply(torch.tensor(b0 + e), case_)
    ym = AirfoilCoefficients.apply(torch.tensor(b0 - e), case_)
    fd = float(((yp[0] - 3.0 * yp[1]) - (ym[0] - 3.0 * ym[1])) / (2 * h))
    assert abs(float(b.grad[0]) - fd) <= 1e-6 * abs(fd), (float(b.grad[0]), fd)
    assert torch.all(torch.isfinite(b.grad)) and float(torch.abs(b.grad).max()) > 0.0
