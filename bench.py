#!/usr/bin/env python
"""Benchmark: grid-point-iterations/s of the miniSMAC2D pseudo-time iteration on GB300.

Workload: steady incompressible RANS (artificial compressibility, SA model) around a NACA 4412
airfoil on a synthetic 1921x481 C-grid (the reference's grid family scaled up: wall spacing
1e-5 chord, far field at 10 chords), alpha = 5 deg, Re = 1e6, beta = 10, dtau = 0.1,
underr = 0.01.  A step is one pseudo-time iteration over the whole grid (SA model, residual and
implicit operator assembly, boundary conditions, 2 j- and 2 k-sweeps of block line relaxation,
update, force integration).

The headline (``value``, ``e2e``, ``roofline``) is the plain FP64 path in the reference's
Gauss-Seidel line order (``--mode reference``), whose per-iteration residuals match the
reference's.  The same line carries the two other forms measured in the same run (``modes``):
FP64 in zebra line order, and the FP32 implicit operator inside the FP64 defect correction, and
the time to a 1e-10 residual drop of the plain FP64 and the FP32-preconditioned forms on a case
whose steady state exists (``time_to_1e-10``).

Prints one JSON line.  ``--impl reference`` times the CPU reference of the same iteration (the
C restatement of the Fortran solver under oracle/; the Fortran itself cannot be compiled on
these machines) on the host cores instead.

Multi-GPU: independent replicas (one subgrid per GPU, no collective on the data path); ranks
come from torchrun's environment, the barrier and the max over ranks use gloo on the host.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic traffic per grid point and iteration, by stage, in bytes: each stage reads its
# input fields once and writes its outputs once.  FP64 line relaxation (impsch 1): 405 doubles.
ALG_BYTES = {
    "fp64": {
        "sa": 8 * (14 + 16 + 4),   # SA assembly, 2 scalar sweeps, update + eddy viscosity
        "assemble": 8 * 56,        # q, metrics, dj -> s and 45 block entries
        "resid": 8 * 4,            # s, dj
        "factor_j": 8 * 45, "sweep_j": 8 * 108, "undo_j": 8 * 45,
        "factor_k": 8 * 45, "sweep_k": 8 * 108,
        "update": 8 * 9,
    },
    # LU-SGS (impsch 2): factored diagonal 18, forward sweep 33, diagonal multiply 15, backward
    # sweep 33 doubles per point, all in the factor_j stage of the stage profile
    "lusgs": {
        "sa": 8 * 32, "assemble": 8 * 56, "resid": 8 * 4, "factor_j": 8 * (18 + 33 + 15 + 33), "update": 8 * 9,
    },
    # FP32 blocks, factors and dq; FP64 q, s, metrics and the SA model
    "mixed": {
        "sa": 8 * 34, "assemble": 8 * 8 + 8 * 3 + 4 * 45, "resid": 8 * 4,
        "factor_j": 4 * 45, "sweep_j": 2 * (8 * 3 + 4 * 45 + 4 * 3 + 4 * 3), "undo_j": 0,
        "factor_k": 4 * 45, "sweep_k": 2 * (8 * 3 + 4 * 45 + 4 * 3 + 4 * 3),
        "update": 8 * 6 + 4 * 3,
    },
}
MODES = {
    "reference": dict(order=0, precision=0),   # the reference's Gauss-Seidel line order, FP64
    "multicolor": dict(order=1, precision=0),  # zebra line order, FP64
    "mixed": dict(order=1, precision=1),       # zebra line order, FP32 operator, FP64 residual/update
}
MODE_TEXT = {"reference": "FP64 plain path, reference Gauss-Seidel line order",
             "multicolor": "FP64, zebra line order",
             "mixed": "FP32 implicit operator in FP64 defect correction, zebra line order"}


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel_prefix: str, workload: str):
    """DRAM bytes per launch of a kernel from the committed ncu summary (profiles/), if one
    exists for this workload: (bytes, source) or (None, None)."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as fh:
            d = json.load(fh)
        for rec in d.get("kernels", []):
            if rec["kernel"].startswith(kernel_prefix) and rec.get("workload") == workload:
                return float(rec["dram_bytes_per_launch"]), rec.get("source")
    except Exception:
        pass
    return None, None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix=f"smac_clocks_gpu{self.gpu}_", suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc:
            return None
        rows = []
        try:
            with open(self.path) as fh:
                lines = fh.readlines()
            os.unlink(self.path)
            for line in lines:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload_params(args, mode=None):
    from minismac_gb300 import abi
    m = MODES[mode or args.mode]
    return abi.default_params(alpha=5.0, beta=10.0, reynum=1.0e6, dtau=0.1, underr=0.01, impsch=args.impsch, **m)


def workload_name(args, mode=None):
    mode = mode or args.mode
    scheme = "block line relaxation" if args.impsch == 1 else "LU-SGS"
    return (f"NACA4412 C-grid {args.jmax}x{args.kmax}, alpha 5, Re 1e6, steady RANS + SA, "
            f"{MODE_TEXT[mode] if args.impsch == 1 else 'FP64 plain path'}, {scheme}")


def config_dict(args):
    return {
        "workload": workload_name(args),
        "mode": args.mode,
        "grid_points": args.jmax * args.kmax,
        "alpha_deg": 5.0, "reynolds": 1.0e6, "beta": 10.0, "dtau": 0.1, "underr": 0.01,
        "sweeps": "2 j + 2 k (mean flow), 2 j (SA)" if args.impsch == 1 else "ILU(0) forward + backward",
        "l2": "inputs larger than L2 (working set ~1 GB at 1921x481); no flush needed",
        "parallelism": "replicas",
    }


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_sample(args, seconds_budget: float, threads: int = 1):
    """Time the oracle on the same workload with `threads` OpenMP threads on the loops the
    reference parallelises: one untimed iteration (wall distance included), then whole
    iterations until the budget is spent."""
    from minismac_gb300 import inputs
    from oracle.oracle_py import Oracle
    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    o = Oracle(workload_params(args), g, rows)
    o.set_threads(threads)
    o.step()
    n, t0 = 0, time.perf_counter()
    while True:
        o.step()
        n += 1
        if time.perf_counter() - t0 > seconds_budget or n >= 50:
            break
    dt = time.perf_counter() - t0
    o.close()
    return n, dt


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference on the host cores (rank 0)."""
    if rank != 0:
        return 0
    from minismac_gb300 import inputs
    from oracle.oracle_py import Oracle
    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    o = Oracle(workload_params(args), g, rows)
    threads = host_threads()
    o.set_threads(threads)
    for _ in range(args.warmup):
        o.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step()
    dt = time.perf_counter() - t0
    o.close()
    pts = args.jmax * args.kmax
    val = pts * args.steps / dt
    line = {
        "metric": "grid-pt-iters/s", "value": val, "unit": "grid-pt-iters/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_dict(args),
        "cpu_baseline": {"value": val, "unit": "grid-pt-iters/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full iterations of the {args.jmax}x{args.kmax} workload after "
                                   f"{args.warmup} untimed ones; C restatement of the Fortran reference, "
                                   f"gcc -O2 -ffp-contract=off -fopenmp, {threads} threads on the loops the "
                                   "reference parallelises with OpenMP (its Fortran cannot be compiled here: "
                                   "no Fortran compiler)"},
        "e2e": {"value": val, "unit": "grid-pt-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(x: float, world: int) -> float:
    """The slowest replica's time (every rank gets it); gloo on the host."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(points: int, steps: int, ms: float, world: int) -> float:
    """Whole-job grid-pt-iters/s: every replica iterates its own copy of the workload."""
    return world * points * steps / (ms / 1e3)


def iteration_flops(mode: str, impsch: int):
    """FP64 floating-point operations per grid point and iteration (2 per fused multiply-add),
    from the committed ncu instruction counts (profiles/fp64_flops.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_flops.json")) as fh:
            d = json.load(fh)
        rec = d["forms"][f"{mode}/impsch{impsch}"]
        return {"per_point": float(rec["fp64_flops_per_point"]), "source": d["source"]}
    except Exception:
        return None


def fp64_peak_tflops():
    """FP64 dense rate of this GPU measured with cuBLAS (torch float64 matmul, 4096^3, best of
    5), the FP64 roof the line solves are held against."""
    try:
        import torch
        n = 4096
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        for _ in range(2):
            torch.matmul(a, b)
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * n ** 3 / (best / 1e3) / 1e12
    except Exception:
        return None


def measure_mode(args, mode, world, barrier, gpu_index, headline):
    """Timed iterations of one form of the iteration on the bench workload; device time from
    CUDA events on the solver's stream, max over ranks."""
    import numpy as np
    from minismac_gb300 import inputs
    from minismac_gb300.solver import Solver

    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    pts = args.jmax * args.kmax
    t_create = time.perf_counter()
    s = Solver(workload_params(args, mode), g, rows)  # metric, initial state, wall distance, autotune
    create_s = time.perf_counter() - t_create
    s.run(args.warmup)
    launches = s.launches_per_iter()
    barrier()
    clocks = None
    if headline:
        with ClockSampler(gpu_index) as clk:
            s.run(args.steps)  # synchronises; device time from CUDA events on the library's stream
        clocks = clk.summary()
    else:
        s.run(args.steps)
    dev_ms = s.last_run_ms()
    barrier()
    dev_ms = max_over_ranks(dev_ms, world)
    out = {"value": aggregate_rate(pts, args.steps, dev_ms, world), "ms_per_step": dev_ms / args.steps,
           # the reference's own timer also covers setup and the first-call wall distance
           "reference_equivalent": {"value": world * pts * args.steps / (create_s + dev_ms / 1e3),
                                    "setup_s": create_s, "iterations": args.steps},
           "gpu_launches": (launches + 1) * args.steps, "clocks": clocks}

    # stage profile of one iteration (events on the solver's stream) -> dominant stage
    prof = s.profile_iteration()
    out["stage_ms"] = prof
    dom = max(prof, key=prof.get)
    table = ALG_BYTES["mixed" if mode == "mixed" else "fp64"]
    # per launch of the stage's main kernel: a sweep stage is two sweep launches
    nlaunch = 2 if dom in ("sweep_j", "sweep_k") else 1
    alg_bytes = table[dom] * pts / nlaunch
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (prof[dom] / nlaunch / 1e3) / 1e9
    kernel = {"sweep_k": "k_gs_sweep_rows", "sweep_j": "k_gs_sweep_rows", "factor_j": "k_btlu",
              "factor_k": "k_btlu", "sa": "k_sa", "assemble": "k_conup"}.get(dom, dom)
    if mode != "reference":
        kernel = {"sweep_k": "k_zebra", "sweep_j": "k_zebra"}.get(dom, kernel)
    traffic, tsrc = ncu_traffic(kernel, workload_name(args, mode))
    flops = iteration_flops(mode, args.impsch)
    if flops:
        fl = flops["per_point"] * pts
        out["fp64"] = {"flops_per_iteration": fl, "achieved_tflops": fl / (dev_ms / args.steps / 1e3) / 1e12,
                       "source": flops["source"]}
    out["roofline"] = {"bound": "hbm", "kernel_stage": dom, "kernel": kernel, "achieved": achieved,
                       "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                       else "fallback", "traffic": traffic, "traffic_source": tsrc,
                       "alg_bytes_per_launch": alg_bytes, "launches_in_stage": nlaunch,
                       "launch_ms": prof[dom] / nlaunch,
                       "iteration_alg_GBps": sum(table.values()) * pts / (dev_ms / args.steps / 1e3) / 1e9}
    if dom in ("sweep_k", "sweep_j") and mode == "reference":
        # the binding roof of the reference-order sweeps: its lines are solved one after another,
        # so a launch lasts (lines) x (the chain of one line); the cycles at the sampled SM clock
        nl = args.jmax if dom == "sweep_k" else args.kmax
        mhz = (clocks or {}).get("sm_mhz") or 2070.0
        us = prof[dom] / nlaunch * 1e3 / nl
        out["roofline"]["binding"] = "FP64 issue along the chain of dependent line solves (not HBM)"
        out["roofline"]["line_chain"] = {"lines_per_launch": nl, "us_per_line": us, "cycles_per_line": us * mhz,
                                         "sm_mhz": mhz}

    # end to end through the C ABI with host buffers: the caller's q and SA variable go in, q,
    # SA variable and eddy viscosity come back, every step (a Fortran host calling step)
    try:
        import torch
        qh = torch.empty(3 * pts, dtype=torch.float64, pin_memory=True).numpy()
        th = torch.empty(pts, dtype=torch.float64, pin_memory=True).numpy()
        vh = torch.empty(pts, dtype=torch.float64, pin_memory=True).numpy()
        pinned = True
    except Exception:
        qh, th, vh = np.empty(3 * pts), np.empty(pts), np.empty(pts)
        pinned = False
    s.get_state(qh, th, vh)
    ne2e = args.steps
    barrier()
    t0 = time.perf_counter()
    for _ in range(ne2e):
        s.set_state(qh, th)
        s.step()
        s.get_state(qh, th, vh)
    e2e_s = time.perf_counter() - t0
    out["e2e"] = {"value": world * pts * ne2e / e2e_s, "unit": "grid-pt-iters/s",
                  "h2d_bytes_per_step": 8 * 4 * pts, "d2h_bytes_per_step": 8 * 5 * pts + 128,
                  "pinned": pinned, "steps": ne2e}
    s.close()
    return out


def converge(s, target, l2_drop, max_iters, chunk=500):
    """Run a solver in chunks until resmax/resmax0 <= target and the L2 residual has dropped by
    l2_drop from its first iteration (or max_iters): for each criterion the first iteration that
    meets it, the device time up to it, and Cl, Cd there."""
    import numpy as np
    dev_ms, it, l2_0, h = 0.0, 0, None, None
    hits = {"rmax": None, "l2": None}
    t0 = time.perf_counter()
    while it < max_iters and (hits["rmax"] is None or hits["l2"] is None):
        h = s.run(chunk)
        ms = s.last_run_ms()
        if l2_0 is None:
            l2_0 = float(h["rhsnorm"][0])
        for key, arr in (("rmax", h["rmax"] <= target), ("l2", h["rhsnorm"] <= l2_drop * l2_0)):
            w = np.where(arr)[0]
            if hits[key] is None and len(w):
                k = int(w[0])
                hits[key] = {"iterations": it + k + 1, "device_s": (dev_ms + ms * (k + 1) / chunk) / 1e3,
                             "cl": float(h["cl"][k]), "cd": float(h["cd"][k])}
        dev_ms += ms
        it += chunk
    return {"rmax_target": hits["rmax"], "l2_drop_target": hits["l2"], "iterations_run": it,
            "ms_per_iter": dev_ms / it, "wall_s": time.perf_counter() - t0, "rmax_last": float(h["rmax"][-1]),
            "l2_drop_last": float(h["rhsnorm"][-1]) / l2_0, "cl": float(h["cl"][-1]), "cd": float(h["cd"][-1])}


def time_to_drop(args):
    """Iterations and device time until resmax/resmax0 <= conv_target (and until the L2 residual
    has dropped by conv_l2_drop) for the plain FP64 path in the reference's line order, the FP64
    zebra order and the FP32-operator form, on a case with a steady state (laminar Re = 1000:
    with the reference's laminar mean flow, Re = 1e6 has none).  Mixed against zebra isolates
    the share of the FP32 operator; zebra against the reference order that of the line order."""
    from minismac_gb300 import abi, inputs
    from minismac_gb300.solver import Solver
    jm, km = (int(v) for v in args.conv_grid.split("x"))
    g, rows = inputs.naca4_cgrid(jm, km)
    res = {"case": f"NACA4412 C-grid {jm}x{km}, alpha 5, Re 1000 (laminar), beta 10, dtau {args.conv_dtau:g}, "
                   f"underr {args.conv_underr:g}, line relaxation; targets resmax/resmax0 <= {args.conv_target:g} "
                   f"and an L2 residual drop of {args.conv_l2_drop:g}", "forms": {}}
    for mode in args.conv_modes.split(","):
        p = abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=args.conv_dtau, underr=args.conv_underr,
                               **MODES[mode])
        s = Solver(p, g, rows)
        try:
            r = converge(s, args.conv_target, args.conv_l2_drop, args.conv_max_iters)
        except Exception as exc:  # a form that diverges on this case is reported, not fatal
            res["forms"][mode] = {"rmax_target": None, "l2_drop_target": None, "error": str(exc)}
            s.close()
            continue
        hit = r["rmax_target"]
        # the fields the earlier bench lines carried, for the rmax target
        r.update({"iterations": hit and hit["iterations"], "device_s": hit and hit["device_s"]})
        res["forms"][mode] = r
        s.close()
    f = res["forms"]

    def ratio(a, b, key):
        ha, hb = f.get(a, {}).get(key), f.get(b, {}).get(key)
        return ha["device_s"] / hb["device_s"] if ha and hb else None

    for key in ("rmax_target", "l2_drop_target"):
        res[f"speedup_{key}"] = {"mixed_vs_plain_fp64": ratio("reference", "mixed", key),
                                 "mixed_vs_fp64_zebra": ratio("multicolor", "mixed", key),
                                 "fp64_zebra_vs_plain_fp64": ratio("reference", "multicolor", key)}
    if f.get("reference", {}).get("rmax_target") and f.get("mixed", {}).get("rmax_target"):
        a, b = f["reference"]["rmax_target"], f["mixed"]["rmax_target"]
        res["speedup_mixed_vs_plain_fp64"] = a["device_s"] / b["device_s"]
        res["mixed_vs_plain_fp64"] = {"dcl": abs(b["cl"] - a["cl"]), "dcd": abs(b["cd"] - a["cd"])}
    return res


def cpu_time_to_drop(args):
    """CPU baseline of the time-to-drop measurement: the oracle (the reference's algorithm,
    line relaxation in its Gauss-Seidel order, one thread) on the same case until
    resmax/resmax0 <= conv_target, wall-clock; its Cl and Cd there are the FP64 reference values the
    GPU forms are compared with."""
    import numpy as np
    from minismac_gb300 import abi, inputs
    from oracle.oracle_py import Oracle
    jm, km = (int(v) for v in args.conv_grid.split("x"))
    g, rows = inputs.naca4_cgrid(jm, km)
    o = Oracle(abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=args.conv_dtau, underr=args.conv_underr,
                                  impsch=1), g, rows)
    it, hit, t_hit, h = 0, None, None, None
    t0 = time.perf_counter()
    while it < args.conv_max_iters:
        h = o.run(500)
        w = np.where(h["rmax"] <= args.conv_target)[0]
        if len(w):
            hit = it + int(w[0]) + 1
            t_hit = (time.perf_counter() - t0) * (it + w[0] + 1) / (it + 500)
            break
        it += 500
    o.close()
    k = int(w[0]) if hit else -1
    return {"iterations": hit, "wall_s": t_hit, "threads": 1, "cl": float(h["cl"][k]), "cd": float(h["cd"][k])}


STAGE_FORMS = [("FP64 line relaxation, reference order", "reference", 1, "fp64"),
               ("FP64 LU-SGS", "reference", 2, "lusgs"),
               ("FP64 line relaxation, zebra order", "multicolor", 1, "fp64"),
               ("FP32 operator in FP64 defect correction, zebra order", "mixed", 1, "mixed")]


def stage_table(args):
    """Device time of every stage of one iteration (CUDA events at the stage boundaries, the SA
    model in line), the stage's algorithmic bytes (each stage reads its inputs once and writes
    its outputs once) and the achieved GB/s against the measured copy bandwidth, for the four
    forms on the bench workload; median of five profiled iterations after the warm-up."""
    import numpy as np
    from minismac_gb300 import abi, inputs
    from minismac_gb300.solver import Solver
    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    pts = args.jmax * args.kmax
    peak, peak_kind = measured_peaks()
    out = {"workload": f"NACA4412 C-grid {args.jmax}x{args.kmax}, alpha 5, Re 1e6, beta 10, dtau 0.1, underr 0.01",
           "peak_gbs": peak, "peak_source": peak_kind, "forms": {}}
    for name, mode, imp, table in STAGE_FORMS:
        p = abi.default_params(alpha=5.0, beta=10.0, reynum=1.0e6, dtau=0.1, underr=0.01, impsch=imp, **MODES[mode])
        s = Solver(p, g, rows)
        s.run(args.warmup)
        s.run(args.steps)
        ms_iter = s.last_run_ms() / args.steps
        profs = [s.profile_iteration() for _ in range(5)]
        s.close()
        alg = ALG_BYTES[table]
        stages = {}
        for st in profs[0]:
            ms = float(np.median([pr[st] for pr in profs]))
            if ms <= 0.0:
                continue
            b = alg.get(st, 0) * pts
            gbs = b / (ms / 1e3) / 1e9 if b else None
            stages[st] = {"ms": ms, "alg_bytes": b, "GBps": gbs, "frac": gbs / peak if gbs else None}
        tot_b = sum(alg.values()) * pts
        out["forms"][name] = {"ms_per_iteration": ms_iter, "stages": stages,
                              "iteration_alg_GBps": tot_b / (ms_iter / 1e3) / 1e9}
    return out


def config3(args):
    """The FP32-operator configuration: NACA 4412 at alpha 8, Re 3e6 on the 1921x481 C-grid,
    run a fixed number of iterations in the plain FP64 path (reference line order), FP64 zebra
    order and FP32 operator: per form the time per iteration and the final Cl, Cd, and the
    differences of p, u, v, the SA variable, Cl and Cd between the forms (mixed against plain
    FP64, mixed against FP64 zebra: the share of the FP32 operator alone)."""
    import numpy as np
    from minismac_gb300 import abi, inputs
    from minismac_gb300.solver import Solver
    g, rows = inputs.naca4_cgrid(1921, 481)
    N = g.jmax * g.kmax
    n = args.config3
    res = {"case": f"NACA4412 C-grid 1921x481, alpha 8, Re 3e6, beta 10, dtau 0.1, underr 0.01, {n} iterations "
                   "from the free-stream start", "forms": {}}
    states = {}
    for mode in ("reference", "multicolor", "mixed"):
        p = abi.default_params(alpha=8.0, beta=10.0, reynum=3.0e6, dtau=0.1, underr=0.01, **MODES[mode])
        s = Solver(p, g, rows)
        dev_ms, h = 0.0, None
        done = 0
        while done < n:
            k = min(500, n - done)
            h = s.run(k)
            dev_ms += s.last_run_ms()
            done += k
        states[mode] = (s.get("q"), s.get("anut"), float(h["cl"][-1]), float(h["cd"][-1]))
        res["forms"][mode] = {"ms_per_iter": dev_ms / n, "cl": float(h["cl"][-1]), "cd": float(h["cd"][-1]),
                              "rmax": float(h["rmax"][-1]), "rhsnorm": float(h["rhsnorm"][-1])}
        s.close()

    def diff(a, b):
        qa, aa, cla, cda = states[a]
        qb, ab, clb, cdb = states[b]
        d = {name: float(np.abs(qa[i * N:(i + 1) * N] - qb[i * N:(i + 1) * N]).max()) for i, name in enumerate("puv")}
        d["nu_tilde_rel"] = float(np.abs(aa - ab).max() / max(np.abs(ab).max(), 1e-300))
        d["cl"], d["cd"] = abs(cla - clb), abs(cda - cdb)
        return d

    res["mixed_vs_plain_fp64"] = diff("mixed", "reference")
    res["mixed_vs_fp64_zebra"] = diff("mixed", "multicolor")
    res["fp64_zebra_vs_plain_fp64"] = diff("multicolor", "reference")
    return res


BATCH_SIZES = [(119, 31), (241, 61), (481, 121), (961, 241)]


def batch_cases(n: int, seed: int = 20261203):
    """The batched workload: seeded NACA 4-digit airfoils (camber 0-6 %, camber position
    0.2-0.6, thickness 8-18 %), alpha uniform in -4..12 deg, Re log-uniform in 5e5..5e6, C-grid
    sizes drawn from 119x31, 241x61, 481x121, 961x241."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        m, pos, t = rng.uniform(0.0, 0.06), rng.uniform(0.2, 0.6), rng.uniform(0.08, 0.18)
        alpha = rng.uniform(-4.0, 12.0)
        re = 10.0 ** rng.uniform(np.log10(5e5), np.log10(5e6))
        size = BATCH_SIZES[int(rng.integers(0, len(BATCH_SIZES)))]
        out.append(dict(m=m, p=pos, t=t, alpha=alpha, reynum=re, size=size))
    return out


def batched(args):
    """All cases advanced together (one graph launch per iteration of all cases) against the
    same cases advanced one after another; mixed precision.  Three layouts of the batch graph:
    each case's whole iteration on its own branch (autotuned line shapes); the line solves of
    all cases packed into one launch per sweep colour (2 or 4 warps per line); the line sweeps
    of all cases (every colour, the wake-cut injections) in one persistent launch fed by one
    work queue (2 or 4 warps per line item)."""
    from minismac_gb300 import abi, inputs
    from minismac_gb300.solver import Batch, Solver
    cases = batch_cases(args.batch)
    solvers = []
    for c in cases:
        g, rows = inputs.naca4_cgrid(c["size"][0], c["size"][1], m=c["m"], p=c["p"], t=c["t"])
        solvers.append(Solver(abi.default_params(alpha=c["alpha"], beta=10.0, reynum=c["reynum"], dtau=0.1,
                                                 underr=0.01, **MODES["mixed"]), g, rows))
    pts = sum(c["size"][0] * c["size"][1] for c in cases)
    tuned = [s.autotune() for s in solvers]
    k = max(args.steps, 5)
    for s in solvers:  # one after another
        s.run(args.warmup)
    seq_ms = 0.0
    for s in solvers:
        s.run(k)
        seq_ms += s.last_run_ms()
    b = Batch(solvers)
    b.run(args.warmup)
    hist = b.run(k)
    conc_ms = b.last_run_ms()
    finite = all(all(abs(v) < 1e300 for v in h["rhsnorm"]) for h in hist)
    b.close()
    packed = {}
    for wpl in (2, 4):  # the same cases with the line solves of all cases packed per sweep colour
        bp = Batch(solvers, packed=True, warps_per_line=wpl)
        bp.run(args.warmup)
        hp = bp.run(k)
        ms = bp.last_run_ms()
        finite = finite and all(all(abs(v) < 1e300 for v in h["rhsnorm"]) for h in hp)
        bp.close()
        packed[f"{wpl}_warps_per_line"] = {"value": pts * k / (ms / 1e3), "ms_per_iteration": ms / k}
    queue = {}
    for wpl in (2, 4):  # the line sweeps of all cases in one persistent launch
        bq = Batch(solvers, queue=True, warps_per_line=wpl)
        bq.run(args.warmup)
        hq = bq.run(k)
        ms = bq.last_run_ms()
        finite = finite and all(all(abs(v) < 1e300 for v in h["rhsnorm"]) for h in hq)
        bq.close()
        queue[f"{wpl}_warps_per_line"] = {"value": pts * k / (ms / 1e3), "ms_per_iteration": ms / k}
    tiles = {}
    for c, s in zip(cases, solvers):
        tiles.setdefault(f"{c['size'][0]}x{c['size'][1]}", set()).add(s.assembly_tiles())
    for s in solvers:
        s.close()
    by_size = {f"{j}x{kk}": sum(1 for c in cases if c["size"] == (j, kk)) for j, kk in BATCH_SIZES}
    lpw = {}
    for (j, kk), t in zip([c["size"] for c in cases], tuned):
        lpw.setdefault(f"{j}x{kk}", set()).add(t)
    layouts = {("queue", w): v for w, v in queue.items()}
    layouts.update({("packed", w): v for w, v in packed.items()})
    (kind, wkey), best = min(layouts.items(), key=lambda kv: kv[1]["ms_per_iteration"])
    layout = ("every case's own work on its own branch, the line sweeps of all cases in one persistent launch "
              "fed by one work queue" if kind == "queue" else
              "every case's own work on its own branch, the line solves of all cases packed into one launch "
              "per sweep colour")
    return {"cases": args.batch, "grid_points_total": pts, "by_size": by_size, "iterations": k,
            "form": "FP32 implicit operator in FP64 defect correction, zebra line order",
            "layout": f"one graph launch per iteration; {layout} ({wkey.replace('_', ' ')})",
            "value": best["value"], "unit": "grid-pt-iters/s", "ms_per_iteration": best["ms_per_iteration"],
            "one_after_another": {"value": pts * k / (seq_ms / 1e3), "ms_per_iteration": seq_ms / k},
            "speedup_vs_one_after_another": seq_ms / (best["ms_per_iteration"] * k),
            "packed_lines": packed,
            "line_sweep_queue": queue,
            "assembly_tiles_chosen": {sz: sorted(list(v)) for sz, v in tiles.items()},
            "graph_of_cases": {"value": pts * k / (conc_ms / 1e3), "ms_per_iteration": conc_ms / k},
            "lines_per_warp_chosen": {sz: sorted(list(v)) for sz, v in lpw.items()},
            "all_finite": finite, "seed": 20261203}


TABLE_SIZES = [(119, 31), (481, 121), (1921, 481)]
TABLE_FORMS = {"FP64 line relaxation, reference order": ("reference", 1),
               "FP64 LU-SGS": ("reference", 2),
               "FP32 operator in FP64 defect correction, zebra line relaxation": ("mixed", 1)}


def size_table(args):
    """grid-pt-iters/s of the GPU forms and of the CPU oracle (1 thread and all threads) at the
    three grid sizes of the workload family; GPU: device time of `steps` iterations after the
    warm-up, CPU: whole iterations for a bounded time after one untimed iteration."""
    from minismac_gb300 import abi, inputs
    from minismac_gb300.solver import Solver
    from oracle.oracle_py import Oracle
    rows_out = []
    for jm, km in TABLE_SIZES:
        g, rows = inputs.naca4_cgrid(jm, km)
        pts = jm * km
        entry = {"grid": f"{jm}x{km}", "points": pts, "gpu": {}, "cpu": {}}
        for name, (mode, imp) in TABLE_FORMS.items():
            p = abi.default_params(alpha=5.0, beta=10.0, reynum=1.0e6, dtau=0.1, underr=0.01, impsch=imp,
                                   **MODES[mode])
            s = Solver(p, g, rows)
            s.run(args.warmup)
            s.run(args.steps)
            ms = s.last_run_ms() / args.steps
            s.close()
            entry["gpu"][name] = {"ms_per_iter": ms, "value": pts / (ms / 1e3)}
        for name, imp in (("line relaxation", 1), ("LU-SGS", 2)):
            for threads in (1, host_threads()):
                o = Oracle(abi.default_params(alpha=5.0, beta=10.0, reynum=1.0e6, dtau=0.1, underr=0.01,
                                              impsch=imp), g, rows)
                o.set_threads(threads)
                o.step()
                n, t0 = 0, time.perf_counter()
                while n < 200 and (n < 2 or time.perf_counter() - t0 < 4.0):
                    o.step()
                    n += 1
                dt = time.perf_counter() - t0
                o.close()
                entry["cpu"][f"{name}, {threads} thread{'s' if threads > 1 else ''}"] = {
                    "ms_per_iter": 1e3 * dt / n, "value": pts * n / dt, "iterations": n}
        rows_out.append(entry)
    return {"table": rows_out, "workload": "NACA4412 C-grids, alpha 5, Re 1e6, beta 10, dtau 0.1, underr 0.01"}


def adjoint_bench(args):
    """The differentiation form: converge laminar Re = 1000 on the given grid (a steady state
    exists there; the reference's Re = 1e6 has none), solve the transposed system for Cl and Cd,
    take the gradients for alpha and 16 Hicks-Henne bumps, and check some of them against
    central differences (step 1e-6) of re-converged GPU solves warm-started from the base state.
    Wall-clock times of each phase (host timers around synchronous calls)."""
    from minismac_gb300 import abi, adjoint, design, inputs
    from minismac_gb300.solver import Solver
    jm, km = (int(v) for v in args.adjoint.split("x"))
    g, rows = inputs.naca4_cgrid(jm, km)
    p = abi.default_params(alpha=5.0, beta=10.0, reynum=1000.0, dtau=0.5, underr=1.0, impsch=1, iturb=0,
                           visc_fp64=1, precision=abi.PREC_MIXED, order=abi.ORDER_MULTICOLOR)

    def make(grid, dalpha):
        q = abi.SmacParams.from_buffer_copy(p)
        q.alpha = p.alpha + dalpha
        return Solver(q, grid, rows)

    s = make(g, 0.0)
    t0 = time.perf_counter()
    conv = adjoint.converge(s, max_iter=300000, chunk=2000)
    conv["seconds"] = time.perf_counter() - t0
    d = design.Design(g, rows)
    r = adjoint.gradients(s, d)
    names = [n for n in args.adjoint_fd.split(",") if n]
    t1 = time.perf_counter()
    fd = adjoint.finite_differences(make, d, names, 1e-6, s.get("q"), s.get_clift(), max_iter=300000, chunk=2000)
    fd_s = time.perf_counter() - t1
    check = {}
    for i, n in enumerate(names):
        k = d.names.index(n)
        check[n] = {o: {"adjoint": float(r[o][k]), "fd": float(fd[o][i]),
                        "rel_err": float(abs(r[o][k] - fd[o][i]) / abs(fd[o][i]))} for o in ("cl", "cd")}
    return {"adjoint": {
        "workload": f"NACA4412 {jm}x{km} C-grid, alpha 5, laminar Re 1000, beta 10, dtau 0.5, underr 1, "
                    f"FP64 viscous fluxes; primal: FP32-operator zebra form to the round-off floor",
        "design_variables": d.names, "primal": conv, "prepare_s": r["prepare_s"],
        "solve": {o: r["stats"][o] for o in ("cl", "cd")},
        "gradient": {"cl": r["cl"].tolist(), "cd": r["cd"].tolist()},
        "fd_check": check, "fd_seconds": fd_s, "fd_iterations": fd["iterations"]}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--jmax", type=int, default=1921)
    ap.add_argument("--kmax", type=int, default=481)
    ap.add_argument("--impsch", type=int, default=1)
    ap.add_argument("--mode", default="reference", choices=sorted(MODES), help="the headline form")
    ap.add_argument("--modes", default="multicolor,mixed", help="other forms measured in the same run ('' = none)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--conv-grid", default="119x31", help="grid of the time-to-1e-10 measurement ('' = skip)")
    ap.add_argument("--conv-modes", default="reference,multicolor,mixed")
    ap.add_argument("--conv-target", type=float, default=1e-10, help="resmax/resmax0 target of the time to drop")
    ap.add_argument("--conv-l2-drop", type=float, default=1e-10, help="L2 residual drop target of the time to drop")
    ap.add_argument("--conv-dtau", type=float, default=0.5, help="pseudo-time step of the time-to-drop case")
    ap.add_argument("--conv-underr", type=float, default=1.0, help="under-relaxation of the time-to-drop case")
    ap.add_argument("--conv-max-iters", type=int, default=30000)
    ap.add_argument("--batch", type=int, default=64, help="cases of the batched measurement (0 = skip)")
    ap.add_argument("--table", action="store_true",
                    help="instead of the bench line: GPU forms and the CPU oracle at 119x31, 481x121, 1921x481")
    ap.add_argument("--adjoint", default="", metavar="JxK",
                    help="instead of the bench line: the discrete-adjoint workload on this grid (e.g. 481x121)")
    ap.add_argument("--adjoint-fd", default="alpha,upper_3", help="variables checked by finite differences")
    ap.add_argument("--stage-table", action="store_true",
                    help="instead of the bench line: per-stage device time and algorithmic GB/s of the four forms")
    ap.add_argument("--config3", type=int, default=0, metavar="N",
                    help="instead of the bench line: N iterations at alpha 8, Re 3e6, 1921x481 in the three forms")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, local, world = env_rank()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return rc

    from minismac_gb300 import build
    build.build()
    if args.table:
        if rank == 0:
            print(json.dumps(size_table(args)), flush=True)
        return 0
    if args.adjoint:
        if rank == 0:
            print(json.dumps(adjoint_bench(args)), flush=True)
        return 0
    if args.stage_table:
        if rank == 0:
            print(json.dumps(stage_table(args)), flush=True)
        return 0
    if args.config3:
        if rank == 0:
            print(json.dumps(config3(args)), flush=True)
        return 0

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    gpu_index = local if world > 1 else 0
    head = measure_mode(args, args.mode, world, barrier, gpu_index, headline=True)
    pts = args.jmax * args.kmax
    line = {
        "metric": "grid-pt-iters/s", "value": head["value"], "unit": "grid-pt-iters/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (generated NACA 4412 C-grid; no dataset)", "config": config_dict(args),
        "roofline": head["roofline"], "stage_ms": head["stage_ms"], "e2e": head["e2e"],
        "gpu_launches": head["gpu_launches"], "clocks": head["clocks"],
        "reference_equivalent": head["reference_equivalent"],
    }
    if "fp64" in head:
        peak = fp64_peak_tflops()
        f = dict(head["fp64"])
        f["peak_tflops"] = peak
        f["peak_source"] = "cuBLAS float64 matmul 4096^3 on this GPU, measured in this run"
        f["frac"] = f["achieved_tflops"] / peak if peak else None
        line["fp64_roofline"] = f
    if args.impsch == 1 and args.modes:
        line["modes"] = {}
        for mode in [m for m in args.modes.split(",") if m and m != args.mode]:
            r = measure_mode(args, mode, world, barrier, gpu_index, headline=False)
            line["modes"][mode] = {"workload": workload_name(args, mode), "value": r["value"],
                                   "ms_per_step": r["ms_per_step"], "e2e": r["e2e"]["value"],
                                   "stage_ms": r["stage_ms"], "roofline": r["roofline"],
                                   "gpu_launches": r["gpu_launches"], "fp64": r.get("fp64")}
    if rank == 0 and args.conv_grid:
        line["time_to_1e-10"] = time_to_drop(args)
    if rank == 0 and args.batch > 0:
        line["batched"] = batched(args)
    if rank == 0 and not args.no_cpu:
        threads = host_threads()
        n, dt = cpu_sample(args, args.cpu_seconds, threads)
        n1, dt1 = cpu_sample(args, args.cpu_seconds / 2, 1)
        line["cpu_baseline"] = {"value": pts * n / dt, "unit": "grid-pt-iters/s", "cores": threads, "kind": "port",
                                "sample": f"{n} iterations of the {args.jmax}x{args.kmax} workload after one "
                                          f"untimed iteration; C restatement of the Fortran reference, "
                                          f"gcc -O2 -ffp-contract=off -fopenmp, {threads} threads on the loops "
                                          f"the reference parallelises with OpenMP",
                                "single_core": {"value": pts * n1 / dt1, "iterations": n1}}
        if args.conv_grid:
            ref = cpu_time_to_drop(args)
            line["cpu_baseline"]["time_to_1e-10"] = ref
            conv = line.get("time_to_1e-10", {}).get("forms", {})
            if ref["iterations"]:
                line["time_to_1e-10"]["vs_cpu_reference"] = {
                    m: {"dcl": abs(f["rmax_target"]["cl"] - ref["cl"]), "dcd": abs(f["rmax_target"]["cd"] - ref["cd"]),
                        "speedup": ref["wall_s"] / f["rmax_target"]["device_s"]}
                    for m, f in conv.items() if f.get("rmax_target")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
