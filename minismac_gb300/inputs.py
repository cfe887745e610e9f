"""Input formats of miniSMAC2D and a synthetic NACA 4-digit C-grid generator.

Readers and writers for the three files the reference solver consumes:

* ``smac2d.in``   Fortran namelist ``&input ... $end`` (ref/initia.f:85-89, 118-148);
* ``xy.dat``      formatted PLOT3D-2D grid, optionally with a zone-count header
                  (ref/rgrid.f:50-648, ref/preproc.f:62-130): x(j,k) then y(j,k), j fastest;
* ``bcmain.dat``  boundary-condition rows ``ibcval zone jbeg jend kbeg kend``, comment lines
                  start with ``c``/``C``, tabs are spaces, ``-1``/``-2`` mean max/max-1
                  (ref/rbc.f:255-398).

The grid generator builds the C-grid family used for all synthetic cases: a NACA 4-digit
airfoil (closed trailing edge), the reference's index orientation (j = 1 at the downstream
end of the lower wake, lower surface first, leading edge at the middle index, k = 1 on the
wall / wake cut), wake points that coincide pairwise across the cut, and a geometric normal
spacing from ``ds_wall`` at the wall to a C-shaped far field ``radius`` chords away.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "BCRow",
    "Grid",
    "read_namelist",
    "read_xy",
    "write_xy",
    "read_bcmain",
    "write_bcmain",
    "cgrid_bc_rows",
    "naca4_cgrid",
    "wake_points",
]


# --------------------------------------------------------------------------- namelist
_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eEdD][+-]?\d+)?$")


def _fortran_value(tok: str):
    t = tok.strip().rstrip(",").strip()
    if not t:
        return None
    low = t.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    if (t[0] == "'" and t[-1] == "'") or (t[0] == '"' and t[-1] == '"'):
        return t[1:-1]
    if _NUM.match(t):
        if re.match(r"^[+-]?\d+$", t):
            return int(t)
        return float(low.replace("d", "e"))
    raise ValueError(f"cannot parse namelist value {tok!r}")


def read_namelist(path_or_text: str, group: str = "input") -> dict:
    """Parse the ``&input`` group of smac2d.in into a dict (lower-case keys).

    Supports the subset the reference file uses: one ``name=value`` per entry, ``!``
    comments, quoted strings, Fortran ``d`` exponents, logicals, ``$end`` or ``/``.
    """
    text = path_or_text
    if "\n" not in path_or_text and not path_or_text.lstrip().startswith(("&", "$")):
        with open(path_or_text) as fh:
            text = fh.read()
    out: dict = {}
    inside = False
    for raw in text.splitlines():
        line = raw
        # strip comments outside quotes
        q = None
        for i, ch in enumerate(line):
            if ch in "'\"":
                q = None if q == ch else (ch if q is None else q)
            elif ch == "!" and q is None:
                line = line[:i]
                break
        s = line.strip()
        if not s:
            continue
        low = s.lower()
        if not inside:
            if low.startswith(("&" + group, "$" + group)):
                inside = True
                s = s[len(group) + 1:].strip()
                if not s:
                    continue
            else:
                continue
        if low.startswith(("$end", "&end", "/")):
            break
        if "=" not in s:
            raise ValueError(f"namelist line without '=': {raw!r}")
        name, val = s.split("=", 1)
        out[name.strip().lower()] = _fortran_value(val)
    if not inside:
        raise ValueError(f"namelist group &{group} not found")
    return out


# --------------------------------------------------------------------------- xy.dat
@dataclass
class Grid:
    jmax: int
    kmax: int
    x: np.ndarray  # shape (kmax, jmax) in C order == Fortran x(jmax,kmax) memory order
    y: np.ndarray

    def flat(self):
        """x, y as contiguous float64 vectors in Fortran (j fastest) order."""
        return (np.ascontiguousarray(self.x, dtype=np.float64).ravel(),
                np.ascontiguousarray(self.y, dtype=np.float64).ravel())


def read_xy(path: str) -> Grid:
    """Read a formatted PLOT3D-2D grid (single zone; a leading zone count of 1 is allowed)."""
    with open(path) as fh:
        toks = fh.read().split()
    vals = toks
    # header: [nzone] jmax kmax
    ints = []
    i = 0
    while i < len(vals) and len(ints) < 3 and re.match(r"^[+-]?\d+$", vals[i]):
        ints.append(int(vals[i]))
        i += 1
    if len(ints) == 3:
        nz, jmax, kmax = ints
        if nz != 1:
            raise ValueError("only single-zone grids are supported")
    elif len(ints) == 2:
        jmax, kmax = ints
    else:
        raise ValueError("bad PLOT3D header")
    n = jmax * kmax
    data = np.array([float(v.replace("d", "e").replace("D", "e")) for v in vals[i:i + 2 * n]])
    if data.size != 2 * n:
        raise ValueError("truncated grid file")
    return Grid(jmax, kmax, data[:n].reshape(kmax, jmax), data[n:].reshape(kmax, jmax))


def write_xy(path: str, g: Grid, zone_header: bool = True) -> None:
    x, y = g.flat()
    with open(path, "w") as fh:
        if zone_header:
            fh.write("  1\n")
        fh.write(f"  {g.jmax}    {g.kmax}\n")
        vals = np.concatenate([x, y])
        for i in range(0, vals.size, 5):
            fh.write("".join(f"{v:24.16e}" for v in vals[i:i + 5]) + "\n")


# --------------------------------------------------------------------------- bcmain.dat
@dataclass
class BCRow:
    ibcval: int
    zone: int
    jbeg: int
    jend: int
    kbeg: int
    kend: int


def read_bcmain(path: str) -> list[BCRow]:
    rows: list[BCRow] = []
    with open(path) as fh:
        for raw in fh:
            line = raw.replace("\t", " ").rstrip("\n")
            if not line.strip() or line[:1] in ("c", "C"):
                continue
            parts = line.split()
            if len(parts) < 6:
                raise ValueError(f"bad bcmain.dat row: {raw!r}")
            rows.append(BCRow(*[int(p) for p in parts[:6]]))
    if not rows:
        raise ValueError("no boundary conditions in bcmain.dat")
    return rows


def write_bcmain(path: str, rows: list[BCRow], title: str = "") -> None:
    with open(path, "w") as fh:
        fh.write("c" + "*" * 70 + "\nc\n")
        fh.write(f"c  {title}\n")
        fh.write("c" + "-" * 70 + "\n")
        fh.write("c  ibcval    zone\tjbeg jend\tkbeg kend\n")
        fh.write("c" + "-" * 70 + "\nc\n")
        for r in rows:
            fh.write(f"\t{r.ibcval}\t{r.zone}\t{r.jbeg} {r.jend}\t\t{r.kbeg} {r.kend}\n")


def cgrid_bc_rows(jmax: int, nwake: int) -> list[BCRow]:
    """The C-grid BC set of the shipped 119x31 case (outflow, wall, far field, wake cut),
    for a grid with ``nwake`` wake points per side including the outflow point."""
    jte1, jte2 = nwake + 1, jmax - nwake
    return [
        BCRow(31, 1, 1, 1, 1, -1),
        BCRow(31, 1, -1, -1, 1, -1),
        BCRow(0, 1, jte1, jte2, 1, 1),
        BCRow(25, 1, 2, -2, -1, -1),
        BCRow(60, 1, 2, jte1 - 1, 1, 1),
        BCRow(60, 1, jte2 + 1, -2, 1, 1),
    ]


# --------------------------------------------------------------------------- grid generator
def wake_points(jmax: int) -> int:
    """Wake points per side (including the outflow end) for a C-grid of ``jmax`` points:
    20 of 119 as in the shipped grid, the same fraction for larger grids."""
    return max(3, int(round((jmax - 1) * 20.0 / 118.0)))


def _naca4(xc: np.ndarray, m: float, p: float, t: float):
    yt = 5.0 * t * (0.2969 * np.sqrt(xc) - 0.1260 * xc - 0.3516 * xc**2 + 0.2843 * xc**3 - 0.1036 * xc**4)
    if m == 0.0 or p == 0.0:
        yc = np.zeros_like(xc)
        dyc = np.zeros_like(xc)
    else:
        fwd = xc < p
        yc = np.where(fwd, m / p**2 * (2 * p * xc - xc**2), m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * xc - xc**2))
        dyc = np.where(fwd, 2 * m / p**2 * (p - xc), 2 * m / (1 - p) ** 2 * (p - xc))
    th = np.arctan(dyc)
    xu, yu = xc - yt * np.sin(th), yc + yt * np.cos(th)
    xl, yl = xc + yt * np.sin(th), yc - yt * np.cos(th)
    return xu, yu, xl, yl


def _geometric_ratio(first: float, total: float, n: int) -> float:
    """Ratio r with first*(r**n - 1)/(r - 1) == total (n intervals)."""
    if first * n >= total:
        return 1.0
    lo, hi = 1.0 + 1e-12, 1.0 + 200.0 / n
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        s = first * (mid**n - 1.0) / (mid - 1.0)
        if s > total:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


def naca4_cgrid(jmax: int, kmax: int, m: float = 0.04, p: float = 0.4, t: float = 0.12,
                ds_wall: float = 1e-5, radius: float = 10.0, nwake: int | None = None,
                d_normal: float = 0.02) -> tuple[Grid, list[BCRow]]:
    """Algebraic C-grid around a NACA 4-digit airfoil (defaults: NACA 4412).

    Returns the grid and its bcmain.dat rows.  ``jmax`` must be odd (leading edge at the
    middle index).  Orientation and pairing follow the shipped 119x31 grid.
    """
    if jmax % 2 == 0 or jmax < 11 or kmax < 5:
        raise ValueError("jmax must be odd and >= 11, kmax >= 5")
    nw = wake_points(jmax) if nwake is None else nwake
    jte1, jte2 = nw + 1, jmax - nw          # 1-based trailing-edge indices
    jle = (jmax + 1) // 2
    nside = jle - jte1 + 1                   # points TE..LE per side
    beta = np.linspace(0.0, math.pi, nside)
    xc = 0.5 * (1.0 - np.cos(beta))          # 0 (LE) .. 1 (TE)
    xu, yu, xl, yl = _naca4(xc, m, p, t)
    # inner line (k = 1), 0-based j
    xin = np.zeros(jmax)
    yin = np.zeros(jmax)
    # lower surface: j = jte1..jle  <->  x from TE to LE
    xin[jte1 - 1:jle] = xl[::-1]
    yin[jte1 - 1:jle] = yl[::-1]
    # upper surface: j = jle..jte2  <->  x from LE to TE
    xin[jle - 1:jte2] = xu
    yin[jle - 1:jte2] = yu
    xin[jte1 - 1] = xin[jte2 - 1] = 1.0
    yin[jte1 - 1] = yin[jte2 - 1] = 0.0
    # wake: geometric from the TE spacing out to x = 1 + radius
    dte = math.hypot(xin[jte1] - xin[jte1 - 1], yin[jte1] - yin[jte1 - 1])
    r = _geometric_ratio(dte, radius, nw)
    xw = 1.0 + dte * (r ** np.arange(1, nw + 1) - 1.0) / (r - 1.0)   # nw points downstream of TE
    xw[-1] = 1.0 + radius
    for i in range(nw):
        xin[jte1 - 2 - i] = xw[i]            # lower wake, j = jte1-1 .. 1
        xin[jte2 + i] = xw[i]                # upper wake, j = jte2+1 .. jmax
        yin[jte1 - 2 - i] = 0.0
        yin[jte2 + i] = 0.0
    # outer line (k = kmax): C of semicircle (centre (1,0), radius R) + straight wake legs
    xout = np.zeros(jmax)
    yout = np.zeros(jmax)
    for j in range(jmax):
        if j < jte1 - 1:
            xout[j], yout[j] = xin[j], -radius
        elif j > jte2 - 1:
            xout[j], yout[j] = xin[j], radius
    # arc length along the airfoil surface -> angle on the semicircle
    sx = xin[jte1 - 1:jte2]
    sy = yin[jte1 - 1:jte2]
    arc = np.concatenate([[0.0], np.cumsum(np.hypot(np.diff(sx), np.diff(sy)))])
    s = arc / arc[-1]
    th = -0.5 * math.pi - math.pi * s
    xout[jte1 - 1:jte2] = 1.0 + radius * np.cos(th)
    yout[jte1 - 1:jte2] = radius * np.sin(th)
    # outward unit normals of the inner line (tangent rotated +90 degrees)
    tx = np.empty(jmax)
    ty = np.empty(jmax)
    tx[1:-1] = xin[2:] - xin[:-2]
    ty[1:-1] = yin[2:] - yin[:-2]
    tx[0], ty[0] = xin[1] - xin[0], yin[1] - yin[0]
    tx[-1], ty[-1] = xin[-1] - xin[-2], yin[-1] - yin[-2]
    tn = np.hypot(tx, ty)
    nx, ny = -ty / tn, tx / tn
    # near the trailing edge the lines turn towards the wake-line direction (perpendicular
    # to the cut) so that they cannot cross the trailing-edge and wake lines
    for j in range(jte1 - 1, jte2):
        phi = max(0.0, 1.0 - (1.0 - xin[j]) / 0.2) ** 2
        vy = -1.0 if j < jle - 1 else 1.0
        ax, ay = (1.0 - phi) * nx[j], (1.0 - phi) * ny[j] + phi * vy
        a = math.hypot(ax, ay)
        nx[j], ny[j] = ax / a, ay / a
    # lines: geometric spacing from ds_wall; they leave the wall along the normal and
    # bend towards the far-field point: P = in + d w n + f (1-w) (out - in), f = d / L,
    # w = exp(-d / d_normal): normal to the wall for the first ~d_normal chords
    dist = []
    for j in range(jmax):
        L = math.hypot(xout[j] - xin[j], yout[j] - yin[j])
        rr = _geometric_ratio(ds_wall, L, kmax - 1)
        if rr == 1.0:
            d = np.linspace(0.0, L, kmax)
        else:
            d = ds_wall * (rr ** np.arange(kmax) - 1.0) / (rr - 1.0)
            d[-1] = L
        dist.append((d, L))

    def lines(dn):
        X = np.zeros((kmax, jmax))
        Y = np.zeros((kmax, jmax))
        for j in range(jmax):
            d, L = dist[j]
            f = d / L
            w = np.exp(-d / dn)
            X[:, j] = xin[j] + d * w * nx[j] + f * (1.0 - w) * (xout[j] - xin[j])
            Y[:, j] = yin[j] + d * w * ny[j] + f * (1.0 - w) * (yout[j] - yin[j])
        return X, Y

    # strongly cambered thin sections can fold lines near the leading edge for one blending
    # length: take the first of a few lengths that gives positive cell areas everywhere
    for dn in (d_normal, 0.5 * d_normal, 2.0 * d_normal, 0.25 * d_normal, 4.0 * d_normal):
        X, Y = lines(dn)
        if _cells_positive(X, Y):
            return Grid(jmax, kmax, X, Y), cgrid_bc_rows(jmax, nw)
    raise ValueError(f"no fold-free C-grid for m={m}, p={p}, t={t} at {jmax}x{kmax}")


def _cells_positive(X: np.ndarray, Y: np.ndarray) -> bool:
    """All cells of the (kmax, jmax) grid have positive area (the wake-cut cells included)."""
    a = (X[1:, 1:] - X[:-1, :-1]) * (Y[1:, :-1] - Y[:-1, 1:]) - (X[1:, :-1] - X[:-1, 1:]) * (Y[1:, 1:] - Y[:-1, :-1])
    return bool(np.all(a > 0)) or bool(np.all(a < 0))
