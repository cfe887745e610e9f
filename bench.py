#!/usr/bin/env python
"""Benchmark: grid-point-iterations/s of the miniSMAC2D pseudo-time iteration on GB300.

Workload: steady incompressible RANS (artificial compressibility, SA model) around a NACA 4412
airfoil on a synthetic 1921x481 C-grid (the reference's grid family scaled up: wall spacing
1e-5 chord, far field at 10 chords), alpha = 5 deg, Re = 1e6, beta = 10, dtau = 0.1,
underr = 0.01, FP64, block line relaxation in the reference's Gauss-Seidel line order.
A step is one pseudo-time iteration over the whole grid (SA model, residual and implicit
operator assembly, boundary conditions, 2 j- and 2 k-sweeps, update, force integration).

Prints one JSON line.  ``--impl reference`` times the CPU reference of the same iteration (the
C restatement of the Fortran solver under oracle/, which cannot be built from its Fortran
sources on these machines) on the host cores instead.

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

# algorithmic FP64 traffic per grid point and iteration, by stage, in doubles: each stage reads
# its input fields once and writes its outputs once (line relaxation, impsch = 1)
ALG_DOUBLES = {
    "sa": 14 + 16 + 4,          # SA assembly, 2 scalar sweeps, update + eddy viscosity
    "assemble": 56,            # q, metrics, dj -> s and 45 block entries
    "resid": 4,                # s, dj
    "factor_j": 45, "sweep_j": 108, "undo_j": 45,
    "factor_k": 45, "sweep_k": 108,
    "update": 9,
}
ALG_BYTES_PER_PT = 8 * 405      # the 405 doubles of the full iteration


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


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{gpu_index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
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
            for line in open(self.path):
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


MODES = {
    "reference": dict(order=0, precision=0),   # the reference's Gauss-Seidel line order, FP64
    "multicolor": dict(order=1, precision=0),  # zebra line order, FP64
    "mixed": dict(order=1, precision=1),       # zebra line order, FP32 operator, FP64 residual/update
}


def workload_params(args):
    from minismac_gb300 import abi
    m = MODES[getattr(args, "mode", "reference")]
    return abi.default_params(alpha=5.0, beta=10.0, reynum=1.0e6, dtau=0.1, underr=0.01, impsch=args.impsch, **m)


def config_dict(args):
    return {
        "workload": f"NACA4412 C-grid {args.jmax}x{args.kmax}, steady RANS + SA, "
                    + {"reference": "FP64 plain path", "multicolor": "FP64 zebra line order",
                       "mixed": "FP32 operator in FP64 defect correction, zebra line order"}[args.mode] + ", "
                    + ("block line relaxation" + (" (reference Gauss-Seidel line order)" if args.mode == "reference" else "")
                       if args.impsch == 1 else "LU-SGS"),
        "mode": args.mode,
        "grid_points": args.jmax * args.kmax,
        "alpha_deg": 5.0, "reynolds": 1.0e6, "beta": 10.0, "dtau": 0.1, "underr": 0.01,
        "sweeps": "2 j + 2 k (mean flow), 2 j (SA)" if args.impsch == 1 else "ILU(0) forward + backward",
        "l2": "inputs larger than L2: working set ~840 B/point, 0.78 GB at 1921x481",
        "parallelism": "replicas",
    }


def cpu_sample(args, seconds_budget: float):
    """Time the oracle (one CPU core) on the same workload: one untimed iteration (wall distance
    included), then whole iterations until the budget is spent."""
    from minismac_gb300 import inputs
    from oracle.oracle_py import Oracle
    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    o = Oracle(workload_params(args), g, rows)
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
    if rank != 0:
        return 0
    from minismac_gb300 import inputs
    from oracle.oracle_py import Oracle
    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    o = Oracle(workload_params(args), g, rows)
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
        "cpu_baseline": {"value": val, "unit": "grid-pt-iters/s", "cores": 1, "kind": "port",
                         "sample": f"{args.steps} full iterations of the {args.jmax}x{args.kmax} workload "
                                   "(the Fortran reference cannot be compiled here: no Fortran compiler)"},
        "e2e": {"value": val, "unit": "grid-pt-iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--jmax", type=int, default=1921)
    ap.add_argument("--kmax", type=int, default=481)
    ap.add_argument("--impsch", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--mode", default="reference", choices=sorted(MODES))
    ap.add_argument("--no-cpu", action="store_true")
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

    import numpy as np
    from minismac_gb300 import build, inputs
    build.build()
    from minismac_gb300.solver import Solver

    g, rows = inputs.naca4_cgrid(args.jmax, args.kmax)
    pts = args.jmax * args.kmax
    s = Solver(workload_params(args), g, rows)
    s.run(args.warmup)
    launches = s.launches_per_iter()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    barrier()
    with ClockSampler(local if world > 1 else 0) as clk:
        s.run(args.steps)  # synchronises; device time from CUDA events on the library's stream
        dev_ms = s.last_run_ms()
    barrier()
    clocks = clk.summary()
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([dev_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
    value = world * pts * args.steps / (dev_ms / 1e3)

    # stage profile of one iteration -> dominant stage and its roofline
    prof = s.profile_iteration()
    dom = max(prof, key=prof.get)
    alg_bytes = ALG_DOUBLES[dom] * 8 * pts
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (prof[dom] / 1e3) / 1e9
    iter_bytes = ALG_BYTES_PER_PT * pts

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
    ne2e = max(1, min(args.steps, 3))
    barrier()
    t0 = time.perf_counter()
    for _ in range(ne2e):
        s.set_state(qh, th)
        s.step()
        s.get_state(qh, th, vh)
    e2e_s = time.perf_counter() - t0
    e2e_val = world * pts * ne2e / e2e_s

    line = {
        "metric": "grid-pt-iters/s", "value": value, "unit": "grid-pt-iters/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_dict(args),
        "roofline": {"bound": "hbm", "kernel_stage": dom, "achieved": achieved, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "alg_bytes_per_launch": alg_bytes,
                     "iteration_alg_GBps": iter_bytes / (dev_ms / args.steps / 1e3) / 1e9},
        "stage_ms": prof,
        "e2e": {"value": e2e_val, "unit": "grid-pt-iters/s", "h2d_bytes_per_step": 8 * 4 * pts,
                "d2h_bytes_per_step": 8 * 5 * pts + 128, "pinned": pinned, "steps": ne2e},
        "gpu_launches": launches * args.steps + args.steps,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        n, dt = cpu_sample(args, args.cpu_seconds)
        line["cpu_baseline"] = {"value": pts * n / dt, "unit": "grid-pt-iters/s", "cores": 1, "kind": "port",
                                "sample": f"{n} iterations of the {args.jmax}x{args.kmax} workload after one "
                                          f"untimed iteration, C oracle -O2 -ffp-contract=off, 1 thread"}
    s.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
