"""GPU parity: the CUDA path against the CPU oracle on the same seeded inputs.

Bit-exact where the arithmetic allows it: the mean-flow assembly, boundary conditions,
factorisations and (with the sequential line solver) whole iterations of p, u, v and the
forces do not depend on transcendental functions, so the GPU reproduces the oracle's bits.
The SA model calls exp, pow and atan, whose CUDA and libm results differ in the last bits:
its arrays are compared with a relative tolerance of 1e-10.  The partitioned line solver
reorders the arithmetic of each line solve: it is compared with the tolerance the
reference's convergence criterion needs (per-iteration L2 residual within 1e-10 relative).
"""
import numpy as np
import pytest

from minismac_gb300 import abi, inputs

pytestmark = pytest.mark.gpu

SA_RTOL = 1e-10


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def make(params, grid, rows):
    from minismac_gb300.solver import Solver
    from oracle.oracle_py import Oracle
    return Solver(params, grid, rows), Oracle(params, grid, rows)


@pytest.fixture(scope="module")
def case119(cuda_lib):
    g, rows = inputs.naca4_cgrid(119, 31)
    return g, rows


def test_setup_bitexact(case119):
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6)
    gpu, orc = make(p, g, rows)
    for name in ("rtxy", "dj", "q"):
        assert np.array_equal(gpu.get(name), orc.get(name)), name
    # the wall distance is computed by the first SA call (ref/tursa.f:131-147)
    gpu.stage_assemble()
    orc.stage_assemble()
    assert np.array_equal(gpu.get("smin"), orc.get("smin"))


@pytest.mark.parametrize("impsch", [1, 2])
def test_assembly_first_step(case119, impsch):
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=impsch)
    gpu, orc = make(p, g, rows)
    og = gpu.stage_assemble()
    oo = orc.stage_assemble()
    # mean-flow residual and blocks: bit-exact
    for name in ("s", "btc", "bjm", "bjp", "bkm", "bkp"):
        a, b = gpu.get(name), orc.get(name)
        assert np.array_equal(a, b), (name, rel(a, b))
    assert (og.jres, og.kres, og.neq_res) == (oo.jres, oo.kres, oo.neq_res)
    assert og.resmax == oo.resmax and og.resmax0 == oo.resmax0 and og.divmax == oo.divmax
    assert abs(og.rhsnorm - oo.rhsnorm) <= 1e-13 * oo.rhsnorm
    # SA state after the SA solve: tolerance (libm vs CUDA transcendental functions)
    assert rel(gpu.get("anut"), orc.get("anut")) < SA_RTOL
    assert rel(gpu.get("vnut"), orc.get("vnut")) < SA_RTOL
    assert abs(og.turres - oo.turres) <= SA_RTOL * abs(oo.turres)


@pytest.mark.parametrize("impsch", [1, 2])
def test_iterations_sequential_bitexact(case119, impsch):
    """Whole iterations with the reference's sequential line arithmetic: p, u, v, Cl, Cd and
    the residual history bit-identical to the oracle."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=impsch,
                           line_solver=abi.LINES_SEQUENTIAL)
    gpu, orc = make(p, g, rows)
    n = 30
    hg, ho = gpu.run(n), orc.run(n)
    for f in ("resmax", "rmax", "divmax", "cd", "cl", "cm", "jres", "kres"):
        assert np.array_equal(hg[f], ho[f]), (f, hg[f][:5], ho[f][:5])
    assert np.abs(hg["rhsnorm"] - ho["rhsnorm"]).max() <= 1e-13 * ho["rhsnorm"].max()
    assert np.array_equal(gpu.get("q"), orc.get("q"))
    assert rel(gpu.get("anut"), orc.get("anut")) < 1e-8


def test_iterations_partitioned(case119):
    """The default (cluster-partitioned) line solver keeps the reference's Gauss-Seidel line
    order; only the carries between line segments are combined by a scan.  Per-iteration L2
    residual within 1e-10 relative of the oracle, Cl / Cd / p, u, v within 1e-9."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=1)
    gpu, orc = make(p, g, rows)
    n = 200
    hg, ho = gpu.run(n), orc.run(n)
    r_l2 = np.abs(hg["rhsnorm"] / ho["rhsnorm"] - 1.0)
    assert r_l2.max() < 1e-10, r_l2.max()
    assert np.abs(hg["resmax"] / ho["resmax"] - 1.0).max() < 1e-9
    for f in ("cl", "cd"):
        assert np.abs(hg[f] - ho[f]).max() < 1e-9 * np.abs(ho[f]).max(), f
    assert rel(gpu.get("q"), orc.get("q")) < 1e-9


@pytest.mark.parametrize("jmax", [721, 1281, 1921, 2001])
def test_iterations_partitioned_long_lines(cuda_lib, jmax):
    """j-lines longer than the 640 segments of one cluster: segments of 2 points (721), of 2
    and 3 points with the line's first point taken out of the scan (1281 = 2 x 640 + 1,
    1921 = 3 x 640 + 1) and of 4 points (2001).  The bounds of the one-point segments, over 20
    iterations."""
    g, rows = inputs.naca4_cgrid(jmax, 31)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=1)
    gpu, orc = make(p, g, rows)
    n = 20
    hg, ho = gpu.run(n), orc.run(n)
    r_l2 = np.abs(hg["rhsnorm"] / ho["rhsnorm"] - 1.0)
    assert r_l2.max() < 1e-10, r_l2.max()
    assert np.abs(hg["resmax"] / ho["resmax"] - 1.0).max() < 1e-9
    for f in ("cl", "cd"):
        assert np.abs(hg[f] - ho[f]).max() < 1e-9 * np.abs(ho[f]).max(), f
    assert rel(gpu.get("q"), orc.get("q")) < 1e-9


def test_sa_short_horizon_reference_config(case119):
    """In the reference configuration the SA model loses its wall distance after the first
    iteration (destruction terms ~1e24), which amplifies last-bit differences of exp / pow /
    atan exponentially; the mean flow does not see the SA variable.  The SA state is therefore
    compared over 10 iterations, where it is still well defined."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=1)
    gpu, orc = make(p, g, rows)
    hg, ho = gpu.run(10), orc.run(10)
    assert rel(gpu.get("anut"), orc.get("anut")) < 1e-10
    assert rel(gpu.get("vnut"), orc.get("vnut")) < 1e-10
    assert np.abs(hg["turres"] / ho["turres"] - 1.0).max() < 1e-10


@pytest.mark.parametrize("impsch", [1, 2])
def test_sa_long_horizon_fixed_wall_distance(case119, impsch):
    """With the wall distance kept on every iteration (labelled deviation) the SA model is
    well conditioned: its state stays within 1e-9 of the oracle over 300 iterations."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=impsch,
                           wall_distance=abi.WALLDIST_FIXED)
    gpu, orc = make(p, g, rows)
    hg, ho = gpu.run(300), orc.run(300)
    assert rel(gpu.get("anut"), orc.get("anut")) < 1e-9
    assert rel(gpu.get("q"), orc.get("q")) < 1e-9
    assert np.abs(hg["cl"] - ho["cl"]).max() < 1e-9 * np.abs(ho["cl"]).max()


def test_stage_lrelax_matches_oracle(case119):
    """smac_lrelax on caller arrays (the reference's lrelax interface) against the oracle's
    lrelax on the same arrays: dq, s (wake-cut rows rewritten) and the restored blocks."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6)
    gpu, orc = make(p, g, rows)
    orc.stage_assemble()
    arrs = {k: orc.get(k) for k in ("q", "s", "btc", "bjm", "bjp", "bkm", "bkp")}
    outs = []
    for solver in (gpu, orc):
        a = {k: v.copy() for k, v in arrs.items()}
        dq = np.zeros_like(a["q"])
        solver.lrelax(a["q"], dq, a["s"], a["btc"], a["bjm"], a["bjp"], a["bkm"], a["bkp"])
        outs.append((dq, a))
    (dg, ag), (do, ao) = outs
    assert rel(dg, do) < 1e-12
    assert rel(ag["s"], ao["s"]) < 1e-12
    for k in ("btc", "bjp", "bkp"):
        assert rel(ag[k], ao[k]) < 1e-12, k


def test_stage_lusgs_matches_oracle(case119):
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=2)
    gpu, orc = make(p, g, rows)
    orc.stage_assemble()
    arrs = {k: orc.get(k) for k in ("q", "s", "btc", "bjm", "bjp", "bkm", "bkp")}
    res = []
    for solver in (gpu, orc):
        a = {k: v.copy() for k, v in arrs.items()}
        dq = np.zeros_like(a["q"])
        scr = np.zeros_like(a["btc"])
        solver.lusgs(3, a["q"], dq, a["s"], a["btc"], a["bjm"], a["bjp"], a["bkm"], a["bkp"], scr)
        res.append((dq, a["s"], scr))
    for x, y in zip(res[0], res[1]):
        assert np.array_equal(x, y)


def _scalar_system(jmax, kmax, seed):
    """Seeded coefficients of the SA model's scalar pentadiagonal system in the reference's
    layout (stc centre, sjm/sjp along j, skm/skp along k), diagonally dominant like the
    assembled ones, with the couplings out of the grid zeroed as the blanking of
    ref/tursa.f:1327-1372 leaves them; a state (turvar) and a right-hand side."""
    rng = np.random.default_rng(seed)
    N = jmax * kmax
    shape = (kmax, jmax)  # j fastest
    stc = 2.0 + rng.random(shape)
    off = {k: -0.45 * rng.random(shape) for k in ("sjm", "sjp", "skm", "skp")}
    off["sjm"][:, 0] = 0.0
    off["sjp"][:, -1] = 0.0
    off["skm"][0, :] = 0.0
    off["skp"][-1, :] = 0.0
    arr = {k: np.ascontiguousarray(v.reshape(N)) for k, v in off.items()}
    arr["stc"] = stc.reshape(N).copy()
    arr["turvar"] = (1e-3 + rng.random(N)) * 1e-2
    arr["rhs"] = rng.standard_normal(N)
    return arr


@pytest.mark.parametrize("line_solver", [abi.LINES_PARTITIONED, abi.LINES_SEQUENTIAL])
def test_stage_lreltur_matches_oracle(case119, line_solver):
    """smac_lreltur on caller arrays (the reference's lreltur(jmax,kmax,turvar,ds,rhs,sjm,sjp,
    skm,skp,stc) interface, ref/lreltur.f:52-160) against the oracle's lreltur on the same
    arrays: ds out, the wake-cut rows of rhs rewritten by the implicit BC injection.  The
    sequential line solver keeps the reference's arithmetic (bit-identical); the partitioned
    one reorders the rounding of each line solve."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, line_solver=line_solver)
    gpu, orc = make(p, g, rows)
    a = _scalar_system(g.jmax, g.kmax, 7)
    res = []
    for solver in (gpu, orc):
        rhs = a["rhs"].copy()
        ds = np.full_like(rhs, 123.0)  # overwritten: lreltur starts from ds = 0
        solver.lreltur(a["turvar"], ds, rhs, a["sjm"], a["sjp"], a["skm"], a["skp"], a["stc"])
        res.append((ds, rhs))
    (dg, rg), (do, ro) = res
    assert not np.array_equal(ro, a["rhs"])  # the wake-cut rows were rewritten
    if line_solver == abi.LINES_SEQUENTIAL:
        np.testing.assert_array_equal(dg, do)
        np.testing.assert_array_equal(rg, ro)
    else:
        assert rel(dg, do) < 1e-13, rel(dg, do)
        assert rel(rg, ro) < 1e-13, rel(rg, ro)


def test_stage_lusgs_scalar_matches_oracle(case119):
    """smac_lusgs with neqs = 1 (the SA model's scalar ILU(0), lusini1 + ilusol1,
    ref/lusgs.f:218-236, ref/ilusol.f:486-591) against the oracle on the same arrays: dq, the
    overwritten rhs and the reciprocal diagonal in scr1, bit-identical (the diagonal order of
    the GPU sweeps computes every point with the reference's operations)."""
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, impsch=2)
    gpu, orc = make(p, g, rows)
    a = _scalar_system(g.jmax, g.kmax, 11)
    res = []
    for solver in (gpu, orc):
        rhs = a["rhs"].copy()
        dq = np.zeros_like(rhs)
        scr = np.zeros_like(rhs)
        solver.lusgs(1, a["turvar"], dq, rhs, a["stc"], a["sjm"], a["sjp"], a["skm"], a["skp"], scr)
        res.append((dq, rhs, scr))
    for name, x, y in zip(("dq", "rhs", "scr1"), res[0], res[1]):
        np.testing.assert_array_equal(x, y, err_msg=name)


def test_throughput_modes_reach_the_reference_fixed_point():
    """Zebra line order (FP64) and the FP32 operator (mixed precision) change the iteration
    history, not the fixed point s = 0: on a converging laminar case (Re = 1000) they end at the
    oracle's Cl, Cd and p, u, v to within the residual level reached, and the FP32 operator
    leaves the zebra history unchanged to 1e-7."""
    from minismac_gb300.solver import Solver
    from oracle.oracle_py import Oracle
    g, rows = inputs.naca4_cgrid(119, 31)
    base = dict(alpha=5.0, beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0)
    n = 6000
    orc = Oracle(abi.default_params(**base), g, rows)
    ho = orc.run(n)
    qo = orc.get("q")
    runs = {}
    for name, kw in (("zebra64", dict(order=abi.ORDER_MULTICOLOR)),
                     ("mixed", dict(order=abi.ORDER_MULTICOLOR, precision=abi.PREC_MIXED))):
        s = Solver(abi.default_params(**base, **kw), g, rows)
        runs[name] = (s.run(n), s.get("q"))
    for name, (h, q) in runs.items():
        assert h["rmax"][-1] < 1e-6, (name, h["rmax"][-1])
        assert abs(h["cl"][-1] - ho["cl"][-1]) < 5e-5, name
        assert abs(h["cd"][-1] - ho["cd"][-1]) < 5e-5, name
        assert np.abs(q - qo).max() < 1e-3, name
    hz, hm = runs["zebra64"][0], runs["mixed"][0]
    # FP32 operator: relative Cl differences at the FP32 level during the transient, shrinking
    # with the correction dq; after 6000 iterations (rmax ~1e-7) within the 1e-8 asked of Cl
    assert (np.abs(hz["cl"] - hm["cl"]) / np.maximum(np.abs(hz["cl"]), 1.0)).max() < 1e-5
    assert abs(hz["cl"][-1] - hm["cl"][-1]) < 1e-8
    assert abs(hm["rmax"][-1] / hz["rmax"][-1] - 1.0) < 0.1


def test_graph_replay_matches_direct_launches(case119, monkeypatch):
    """smac_run replays one captured CUDA graph per iteration; smac_step launches directly.
    Both give the same history."""
    from minismac_gb300.solver import Solver
    g, rows = case119
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6)
    a, b = Solver(p, g, rows), Solver(p, g, rows)
    ha = a.run(20)
    hb = [b.step() for _ in range(20)]
    assert np.array_equal(ha["cl"], np.array([h.cl for h in hb]))
    assert np.array_equal(a.get("q"), b.get("q"))


def test_batch_matches_cases_run_alone(cuda_lib, monkeypatch):
    """Three cases of different grids, airfoils and forms advanced in one graph per iteration
    give each case exactly the history it has when run alone.  The zebra line shapes are fixed:
    the autotuner picks them by timing when a context is created, so two contexts of one case
    could otherwise round their line solves differently."""
    from minismac_gb300.solver import Batch, Solver
    monkeypatch.setenv("SMAC_ZEBRA_SHAPE", "-4,1")
    specs = [((119, 31), dict(m=0.04, p=0.4, t=0.12), dict(alpha=5.0, order=1, precision=1)),
             ((241, 61), dict(m=0.02, p=0.3, t=0.10), dict(alpha=-2.0, order=1, precision=1)),
             ((119, 31), dict(m=0.0, p=0.4, t=0.15), dict(alpha=8.0, order=0, precision=0))]

    def make_cases():
        out = []
        for (jm, km), geo, flow in specs:
            g, rows = inputs.naca4_cgrid(jm, km, **geo)
            out.append(Solver(abi.default_params(beta=10.0, reynum=5e5, **flow), g, rows))
        return out

    alone = [s.run(20) for s in make_cases()]
    cases = make_cases()
    b = Batch(cases)
    together = b.run(20)
    assert b.last_run_ms() > 0
    for ha, hb in zip(alone, together):
        for k in ("resmax", "rhsnorm", "cl", "cd", "turres"):
            np.testing.assert_array_equal(ha[k], hb[k], err_msg=k)
    # a second run continues every case
    more = b.run(5)
    assert all(m["nt"][0] == 21 for m in more)


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_zebra_line_shapes_agree(cuda_lib, monkeypatch, precision):
    """The zebra line solves give the same iterations whatever their shape (1 or 4 lines per
    warp, 2 or 4 warps per line): 10 iterations on 481x121 (j lines of 481 points, k lines of
    121) agree to the rounding of the working precision (segments of different lengths round
    differently; the impulsive start amplifies that)."""
    from minismac_gb300.solver import Solver
    g, rows = inputs.naca4_cgrid(481, 121)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0, iturb=0,
                           order=abi.ORDER_MULTICOLOR, precision=precision)
    res = {}
    for shape in ("1,1", "4,4", "-2,-2", "-4,-4"):
        monkeypatch.setenv("SMAC_ZEBRA_SHAPE", shape)
        s = Solver(p, g, rows)
        assert s.autotune() == tuple(int(v) for v in shape.split(","))
        h = s.run(10)
        res[shape] = (h["rhsnorm"], s.get("q"))
        s.close()
    tol = 1e-10 if precision == abi.PREC_FP64 else 1e-4
    r0, q0 = res["1,1"]
    for shape, (r, q) in res.items():
        assert np.max(np.abs(r - r0) / r0) < tol, shape
        assert np.max(np.abs(q - q0)) < tol, shape


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_assembly_tile_shapes_bitexact(cuda_lib, monkeypatch, precision):
    """The assembly kernels give the same bits whatever their tile shape (the autotuner picks one
    of four per direction by timing): 5 iterations on 241x61 with every shape, the plain
    reference-order path and the FP32-operator form, histories and states identical."""
    from minismac_gb300.solver import Solver
    g, rows = inputs.naca4_cgrid(241, 61)
    order = abi.ORDER_REFERENCE if precision == abi.PREC_FP64 else abi.ORDER_MULTICOLOR
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, order=order, precision=precision)
    monkeypatch.setenv("SMAC_ZEBRA_SHAPE", "-4,1")
    runs = {}
    for shape in ((0, 0), (1, 1), (2, 2), (3, 3)):
        monkeypatch.setenv("SMAC_CONUP_SHAPE", f"{shape[0]},{shape[1]}")
        s = Solver(p, g, rows)
        assert s.assembly_tiles() == shape
        h = s.run(5)
        runs[shape] = (h, s.get("q"), s.get("anut"), s.get("btc"))
        s.close()
    h0, q0, a0, b0 = runs[(0, 0)]
    for shape, (h, q, a, b) in runs.items():
        for key in ("rhsnorm", "resmax", "cl", "cd", "turres"):
            np.testing.assert_array_equal(h[key], h0[key], err_msg=f"{shape} {key}")
        np.testing.assert_array_equal(q, q0)
        np.testing.assert_array_equal(a, a0)
        np.testing.assert_array_equal(b, b0)
    # without a fixed shape the autotuner picks one of the four per direction
    monkeypatch.delenv("SMAC_CONUP_SHAPE")
    s = Solver(p, g, rows)
    assert all(0 <= t < 4 for t in s.assembly_tiles())
    s.close()


@pytest.mark.parametrize("wpl", [2, 4])
def test_queue_batch_matches_packed_batch(cuda_lib, monkeypatch, wpl):
    """The line sweeps of an iteration of every case (every sweep colour of both directions,
    the wake-cut injections) in one persistent launch fed by one work queue give the same
    histories and states, bit for bit, as the packed layout (one launch per colour), on cases
    of five sizes and angles given smallest first (the queue orders them largest first); a
    second run continues every case the same way."""
    from minismac_gb300.solver import Batch, Solver
    monkeypatch.setenv("SMAC_ZEBRA_SHAPE", f"-{wpl},-{wpl}")
    specs = [((79, 21), -3.0), ((119, 31), 2.0), ((241, 61), 6.0), ((119, 31), 9.0), ((481, 121), 4.0)]

    def make():
        out = []
        for (jm, km), a in specs:
            g, rows = inputs.naca4_cgrid(jm, km)
            p = abi.default_params(alpha=a, beta=10.0, reynum=1e6, dtau=0.1, underr=0.01,
                                   order=abi.ORDER_MULTICOLOR, precision=abi.PREC_MIXED)
            out.append(Solver(p, g, rows))
        return out

    runs = []
    for queue in (False, True):
        solvers = make()
        b = Batch(solvers, packed=not queue, queue=queue, warps_per_line=wpl)
        hist = b.run(15) + b.run(5)
        runs.append((hist, [s.get("q") for s in solvers], [s.get("anut") for s in solvers]))
        b.close()
    n = len(specs)
    for i in range(n):
        for key in ("rhsnorm", "resmax", "cl", "cd", "turres", "nt"):
            np.testing.assert_array_equal(runs[0][0][i][key], runs[1][0][i][key], err_msg=f"case {i} {key}")
            np.testing.assert_array_equal(runs[0][0][n + i][key], runs[1][0][n + i][key], err_msg=f"case {i} {key}")
        np.testing.assert_array_equal(runs[0][1][i], runs[1][1][i])
        np.testing.assert_array_equal(runs[0][2][i], runs[1][2][i])


@pytest.mark.parametrize("wpl", [2, 4])
def test_packed_batch_matches_graph_batch(cuda_lib, monkeypatch, wpl):
    """The batch with the line solves of all cases packed into one launch per sweep colour gives
    the same histories, bit for bit, as the batch of per-case branches with the same line shape
    (wpl warps per line), on cases of different sizes and angles."""
    from minismac_gb300.solver import Batch, Solver
    monkeypatch.setenv("SMAC_ZEBRA_SHAPE", f"-{wpl},-{wpl}")
    specs = [((119, 31), 2.0), ((241, 61), 6.0), ((79, 21), -3.0), ((119, 31), 9.0)]

    def make():
        out = []
        for (jm, km), a in specs:
            g, rows = inputs.naca4_cgrid(jm, km)
            p = abi.default_params(alpha=a, beta=10.0, reynum=1e6, dtau=0.1, underr=0.01,
                                   order=abi.ORDER_MULTICOLOR, precision=abi.PREC_MIXED)
            out.append(Solver(p, g, rows))
        return out

    runs = []
    for packed in (False, True):
        solvers = make()
        b = Batch(solvers, packed=packed, warps_per_line=wpl)
        hist = b.run(20)
        runs.append((hist, [s.get("q") for s in solvers]))
        b.close()
    for i in range(len(specs)):
        for key in ("rhsnorm", "resmax", "cl", "cd"):
            np.testing.assert_array_equal(runs[0][0][i][key], runs[1][0][i][key], err_msg=f"case {i} {key}")
        np.testing.assert_array_equal(runs[0][1][i], runs[1][1][i])


@pytest.mark.parametrize("grid", [(481, 121), (1921, 61)])
def test_sa_pivots_warp_per_line_match_sequential(cuda_lib, monkeypatch, grid):
    """The throughput forms factor the SA lines with a warp per line (segment products of the
    pivot recurrence c'_i = c_i / (b_i - a_i c'_{i-1}), scanned across the warp, then each
    segment rerun from its incoming c').  Against the one-thread-per-line factorisation of the
    same scatri arithmetic (ref/lreltur.f:337-359): the same SA iterations to rounding, over 50
    iterations of the FP32-operator form with the wall distance kept (the well-conditioned SA
    configuration), on j-lines of 481 and 1921 points.  The mean-flow line shapes are fixed:
    the autotuner picks them by timing, and two contexts with different shapes would round the
    mean flow, which the SA model reads, differently."""
    from minismac_gb300.solver import Solver
    g, rows = inputs.naca4_cgrid(*grid)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1e6, order=abi.ORDER_MULTICOLOR,
                           precision=abi.PREC_MIXED, wall_distance=abi.WALLDIST_FIXED)
    monkeypatch.setenv("SMAC_ZEBRA_SHAPE", "-2,1")
    res = []
    for sequential in (True, False):
        if sequential:
            monkeypatch.setenv("SMAC_SA_FACTOR_SEQUENTIAL", "1")
        else:
            monkeypatch.delenv("SMAC_SA_FACTOR_SEQUENTIAL", raising=False)
        s = Solver(p, g, rows)
        h = s.run(50)
        res.append((s.get("anut"), h["turres"], s.get("q")))
        s.close()
    (a0, t0, q0), (a1, t1, q1) = res
    assert rel(a1, a0) < 1e-10, rel(a1, a0)
    assert np.max(np.abs(t1 / t0 - 1.0)) < 1e-8
    np.testing.assert_array_equal(q1, q0)  # the SA variable does not feed the mean flow
