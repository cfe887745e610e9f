"""The reference's output formats, written from device state.

- the per-iteration ``XX`` convergence line and its header (ref/smac2d.f:1985-2003,
  FORMAT 100 and 110),
- the PLOT3D function file ``Q2D.p3d`` (ref/smac2d.f:2020-2145, FORMAT 205 and 206): one zone,
  four variables 1, u, v, p/0.4 + (u^2 + v^2)/2 with the reference's single-precision literal
  0.4,
- the YAML run summary (ref/smac2d.f:707-747 header, 2175-2179 airfoil block, 1087-1109 timings).

Fortran edit descriptors are reproduced by ``fortran_e`` / ``fortran_f``; list-directed
output (``write(u,*)``) has no fixed layout in the standard, so the YAML keeps the reference's
keys and order with plain YAML values.
"""
from __future__ import annotations

import datetime as _dt
import getpass
import math
import socket

import numpy as np

F04 = float(np.float32(0.4))  # the REAL*4 literal 0.4 of ref/smac2d.f:2081


def fortran_e(v: float, w: int, d: int, scale: int = 1) -> str:
    """``1PEw.d`` (scale 1): one digit before the point, d after; ``Ew.d`` (scale 0): 0.ddd.
    Exponent E+xx, or +xxx without the letter when |exponent| > 99; right-justified in w
    columns, '*' x w if it does not fit."""
    if not math.isfinite(v):
        s = "NaN" if math.isnan(v) else ("-Infinity" if v < 0 else "Infinity")
        return s.rjust(w) if len(s) <= w else "*" * w
    if v == 0.0:
        mant, ex = ("0." + "0" * d), 0
    elif scale == 1:
        m, e = f"{abs(v):.{d}e}".split("e")
        mant, ex = m, int(e)
    else:  # 0.ddd form: d significant digits
        m, e = f"{abs(v):.{d - 1}e}".split("e")
        mant, ex = "0." + m.replace(".", ""), int(e) + 1
    exp = f"E{ex:+03d}" if abs(ex) <= 99 else f"{ex:+04d}"
    s = ("-" if (v < 0 or (v == 0.0 and math.copysign(1.0, v) < 0)) else "") + mant + exp
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_f(v: float, w: int, d: int, scale: int = 0) -> str:
    """``Fw.d`` (with a ``kP`` scale factor the value is multiplied by 10^k)."""
    x = v * (10.0 ** scale)
    s = f"{x:.{d}f}"
    if s.startswith("-") and float(s) == 0.0:
        s = "-" + s[1:]
    if s.startswith("0.") and len(s) > w:
        s = s[1:]
    elif s.startswith("-0.") and len(s) > w:
        s = "-" + s[2:]
    return s.rjust(w) if len(s) <= w else "*" * w


# ------------------------------------------------------------------------------- XX lines
XX_HEADER = ("\n     nt   resmax     divmax     turres      j     k    nz     cputime       cd          cl\n"
             "   ----  ---------  ---------  ---------  ----  ----  ----  ----------  ----------  ----------")


def xx_header_due(nt: int, ifreq: int = 25) -> bool:
    """The header repeats every ifreq iterations, starting at nt = 1 (ref/smac2d.f:1985-1987)."""
    return ((nt - 1) // ifreq) * ifreq == nt - 1


def xx_line(nt: int, rmax: float, divmax: float, turres: float, jres: int, kres: int, zone: int,
            cputime: float, cd: float, cl: float) -> str:
    """FORMAT 110: ('XX',i5,1p3e11.3,3i6,1p3e12.4)."""
    def i(v, w):
        s = str(int(v))
        return s.rjust(w) if len(s) <= w else "*" * w
    return ("XX" + i(nt, 5) + "".join(fortran_e(v, 11, 3) for v in (rmax, divmax, turres)) +
            "".join(i(v, 6) for v in (jres, kres, zone)) +
            "".join(fortran_e(v, 12, 4) for v in (cputime, cd, cl)))


# ------------------------------------------------------------------------------- Q2D.p3d
def _list_int(*vals) -> str:
    """List-directed integers as gfortran writes them: each in 12 columns."""
    return "".join(f" {int(v):11d}" for v in vals)


def q2d_variables(q: np.ndarray, jmax: int, kmax: int) -> np.ndarray:
    """The four PLOT3D variables (1, u, v, p/0.4 + (u^2 + v^2)/2) as (4, kmax, jmax)."""
    q = np.asarray(q, dtype=np.float64).reshape(3, kmax, jmax)
    pp, uu, vv = q
    out = np.empty((4, kmax, jmax))
    out[0] = 1.0
    out[1] = uu
    out[2] = vv
    out[3] = pp / F04 + 0.5 * (uu * uu + vv * vv)
    return out


def write_q2d(path: str, q: np.ndarray, jmax: int, kmax: int, alpha: float, reynum: float,
              cputime: float) -> None:
    """Write Q2D.p3d for one zone: zone count, jmax kmax, FORMAT 205 (0, alpha, Re, time),
    then the four variables (j fastest, then k, then variable) in FORMAT 206 (6f10.6)."""
    v = q2d_variables(q, jmax, kmax).ravel()
    with open(path, "w") as fh:
        fh.write(_list_int(1) + "\n")
        fh.write(_list_int(jmax, kmax) + "\n")
        fh.write(fortran_f(0.0, 5, 2, scale=1) + " " + " ".join(fortran_e(x, 13, 5) for x in (alpha, reynum, cputime))
                 + "\n")
        for i in range(0, v.size, 6):
            fh.write("".join(fortran_f(x, 10, 6) for x in v[i:i + 6]) + "\n")


def read_q2d(path: str):
    """Read back a Q2D.p3d written by write_q2d: (jmax, kmax, header values, (4, kmax, jmax))."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    nz = int(lines[0])
    if nz != 1:
        raise ValueError("only single-zone files are supported")
    jmax, kmax = (int(t) for t in lines[1].split())
    head = [float(t) for t in lines[2].split()]
    vals = []
    for ln in lines[3:]:
        vals.extend(float(ln[i:i + 10]) for i in range(0, len(ln), 10) if ln[i:i + 10].strip())
    return jmax, kmax, head, np.array(vals).reshape(4, kmax, jmax)


# ------------------------------------------------------------------------------- YAML summary
def yaml_filename(geometry: str, jmax: int, kmax: int, ntmax: int, host: str | None = None,
                  when: _dt.datetime | None = None, ranks: int = 1, threads: int = 0) -> str:
    """smac2d_<geometry>_<host>_<j>x<k>_<ranks>ranks_<threads>threads_<n>iters_double_<date>.yaml
    with blanks of the geometry title replaced by '_' (ref/smac2d.f:666-696)."""
    host = host or socket.gethostname()
    when = when or _dt.datetime.now()
    g = geometry.strip().replace(" ", "_")
    return (f"smac2d_{g}_{host}_{jmax}x{kmax}_{ranks}ranks_{threads}threads_{ntmax}iters_double_"
            f"{when:%Y_%m_%d_%H_%M_%S}.yaml")


def yaml_summary(*, title: str, geometry: str, grid_file: str, jmax: int, kmax: int, beta: float,
                 dtau: float, reynum: float, alpha: float, impsch: int, cd: float, cl: float, cm: float,
                 rmax: float, ntmax: int, init_sec: float, solve_sec: float, filename: str = "",
                 host: str | None = None, when: _dt.datetime | None = None, threads: int = 0) -> str:
    """The reference's YAML keys in its order: run header, airfoil forces and residual (written
    at the last iteration), then the timings."""
    when = when or _dt.datetime.now()
    try:
        user = getpass.getuser()
    except Exception:
        user = "unknown"
    scheme = {1: "line relaxation", 2: "lusgs factorization"}.get(impsch, "unknown")
    per_it = solve_sec / max(ntmax, 1)
    lines = [
        f"user: {user}", "code: smac2d", f"host: {host or socket.gethostname()}",
        f"title: {title.strip()}", f"geometry: {geometry.strip()}",
        f"date_yyyy_mm_dd: {when:%Y_%m_%d}", f"time_of_day: {when:%H_%M_%S}",
        "num_grids: 1", "mpi_ranks: 1", f"num_threads_per_node: {threads}",
        f"total_processes: {threads if threads else 1}",
        f"grid_file: {grid_file}", f"largest_dim: {max(jmax, kmax)}", f"j-dim: {jmax}", f"k-dim: {kmax}",
        f"total_points: {jmax * kmax}", f"beta: {float(beta)!r}", "fp_precision: double",
        f"dtau: {fortran_e(dtau, 12, 4).strip()}", f"reynolds_number: {float(reynum)!r}",
        f"angle_of_attack_degs: {float(alpha)!r}", f"implicit_scheme: {scheme}",
        "airfoil:", f"   cd: {float(cd)!r}", f"   cl: {float(cl)!r}", f"   cm: {float(cm)!r}", f"residual: {float(rmax)!r}",
        f"sec_per_iteration: {fortran_e(per_it, 12, 5).strip()}",
        f"microsec_per_iter_per_point: {fortran_e(per_it / (jmax * kmax) * 1e6, 12, 5).strip()}",
        f"number_of_iterations: {ntmax}", f"alpha_deg: {float(alpha)!r}",
        f"initialize_sec: {fortran_e(init_sec, 12, 5).strip()}", f"send_subgrids_sec: {fortran_e(0.0, 12, 5).strip()}",
        f"solve_sec: {fortran_e(solve_sec, 12, 5).strip()}",
        f"total_time_sec: {fortran_e(init_sec + solve_sec, 12, 5).strip()}",
        f"yaml_filename: {filename}",
    ]
    return "\n".join(lines) + "\n"
