"""The algebra of the partitioned block-tridiagonal line solve, restated in numpy (CPU).

The reference solves each line with the block Thomas algorithm (ref/btlu3.f factorisation,
ref/lrelax.f:225-561 sweeps): y_i = B'_i^-1 (r_i - a_i y_{i-1}), x_i = y_i - c_i x_{i+1}, with
B'_i the factored diagonal block and c_i = B'_i^-1 (upper block).  The partitioned CUDA sweep
splits the line into segments whose recurrences start from a zero carry and are corrected by
the transfer products M_t ... M_1 (forward, M_i = -B'_i^-1 a_i) and (-c_i) ... (backward).  A
line one point longer than a multiple of the segment count takes its first point out of the
scan: the first segment starts from y_1 = z_1 + K r_0 (K = M_1 B'_0^-1) with no carry, and
x_0 = y_0 - c_0 y_1 + c_0 c_1 x_2.  These checks restate that decomposition, not the kernel
(the kernel is compared with the oracle by the GPU tests), on random diagonally dominant lines.
The scalar SA lines' pivots, formed a warp per line by composing segments of the pivot
recurrence (a Moebius map), are restated the same way.
"""
import numpy as np
import pytest


def random_line(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=(n, 3, 3)) * 0.3
    b = rng.normal(size=(n, 3, 3)) * 0.3 + 4.0 * np.eye(3)
    c = rng.normal(size=(n, 3, 3)) * 0.3
    a[0] = 0.0
    c[-1] = 0.0
    r = rng.normal(size=(n, 3))
    return a, b, c, r


def factor(a, b, c):
    """B'_i and c'_i = B'_i^-1 c_i of the block Thomas algorithm."""
    n = len(b)
    Bf = np.empty_like(b)
    cf = np.empty_like(c)
    for i in range(n):
        Bf[i] = b[i] - (a[i] @ cf[i - 1] if i > 0 else 0.0)
        cf[i] = np.linalg.solve(Bf[i], c[i])
    return Bf, cf


def thomas(a, Bf, cf, r):
    n = len(r)
    y = np.empty_like(r)
    for i in range(n):
        y[i] = np.linalg.solve(Bf[i], r[i] - (a[i] @ y[i - 1] if i > 0 else 0.0))
    x = np.empty_like(r)
    for i in reversed(range(n)):
        x[i] = y[i] - (cf[i] @ x[i + 1] if i < n - 1 else 0.0)
    return x


def partitioned(a, Bf, cf, r, L, head):
    """Segments of L points after `head` points taken out of the scan; the carries between
    segments are propagated one segment after the other (the kernel combines them by scans of
    the same transfer operators, which gives the same values up to rounding)."""
    n = len(r)
    Bi = np.array([np.linalg.inv(B) for B in Bf])
    M = np.array([-Bi[i] @ a[i] for i in range(n)])
    z = np.einsum("nij,nj->ni", Bi, r)
    segs = [list(range(s, min(n, s + L))) for s in range(head, n, L)]
    if head:
        K = M[1] @ Bi[0]
        z = z.copy()
        z[1] = z[1] + K @ r[0]           # the first segment starts from y_0 with no carry
    # forward: local pass from a zero carry, then the carry through the segment's transfer
    y = np.zeros_like(r)
    carry = np.zeros(3)
    for k, seg in enumerate(segs):
        yl = np.zeros(3)
        loc = []
        for t, i in enumerate(seg):
            yl = z[i] + (M[i] @ yl if t > 0 else 0.0)
            loc.append(yl)
        T = np.eye(3)
        for t, i in enumerate(seg):
            T = M[i] @ T
            y[i] = loc[t] + T @ carry
        carry = y[seg[-1]]
    # backward
    x = np.zeros_like(r)
    carry = np.zeros(3)
    for seg in reversed(segs):
        xl = np.zeros(3)
        loc = {}
        for t, i in enumerate(reversed(seg)):
            xl = y[i] - (cf[i] @ xl if t > 0 else 0.0)
            loc[i] = xl
        T = np.eye(3)
        for i in reversed(seg):
            T = -cf[i] @ T if i < n - 1 else T * 0.0
            x[i] = loc[i] + T @ carry
        carry = x[seg[0]]
    if head:
        y0 = Bi[0] @ r[0]
        D = cf[0] @ cf[1]
        x[0] = (y0 - cf[0] @ y[1]) + D @ x[2]
    return x


@pytest.mark.parametrize("n,L,head", [(13, 1, 0), (13, 3, 1), (13, 4, 0), (10, 3, 1), (17, 4, 1), (9, 2, 0)])
def test_partitioned_solve_matches_block_thomas(n, L, head):
    a, b, c, r = random_line(n, seed=n * 10 + L + head)
    Bf, cf = factor(a, b, c)
    x_seq = thomas(a, Bf, cf, r)
    x_par = partitioned(a, Bf, cf, r, L, head)
    # and both solve the block-tridiagonal system itself
    A = np.zeros((3 * n, 3 * n))
    for i in range(n):
        A[3 * i:3 * i + 3, 3 * i:3 * i + 3] = b[i]
        if i > 0:
            A[3 * i:3 * i + 3, 3 * i - 3:3 * i] = a[i]
        if i < n - 1:
            A[3 * i:3 * i + 3, 3 * i + 3:3 * i + 6] = c[i]
    x_ref = np.linalg.solve(A, r.ravel()).reshape(n, 3)
    assert np.abs(x_seq - x_ref).max() < 1e-12
    assert np.abs(x_par - x_seq).max() < 1e-12


def direct_carries(a, Bf, cf, r, L, spw, rw, ncta):
    """The partitioned solve of the reference-order CUDA sweep (k_gs_sweep_rows with the operators
    of k_line_prep_rows): segments of L points, spw segments per warp, rw warps per CTA, ncta
    CTAs.  Per direction, every warp scans its segments from a zero carry; a CTA's aggregate is
    the sum of its warps' end values, each through the product of the later warps' transfers;
    after the exchange, every warp forms its carry directly as the sum of its CTA's earlier
    warps' values through Phi(g; k) = W_{g-1}..W_{k+1} and of the earlier CTAs' aggregates
    through K_g Psi(c; c') (K_g = W_{g-1}..W_{4c}, Psi(c; c') = T_{c-1}..T_{c'+1}); the backward
    direction mirrors it on the true forward values."""
    n = len(r)
    I = np.eye(3)
    Bi = np.array([np.linalg.inv(B) for B in Bf])
    M = np.array([-Bi[i] @ a[i] if i > 0 else np.zeros((3, 3)) for i in range(n)])
    H = np.array([-cf[i] if i < n - 1 else np.zeros((3, 3)) for i in range(n)])
    z = np.einsum("nij,nj->ni", Bi, r)
    ns, nw = spw * rw * ncta, rw * ncta
    segs = [list(range(s * L, min(n, s * L + L))) for s in range(ns)]
    assert sum(len(g) for g in segs) == n

    def direction(local, order):
        """local(s) -> (value from a zero carry, transfer) of segment s; order: +1 forward (carry
        from lower indices), -1 backward.  Returns the true incoming carry of every segment."""
        val, T = zip(*[local(s) for s in range(ns)])
        val, T = np.array(val), np.array(T)
        S = np.zeros((ns, 3))          # scanned values inside each warp, zero carry into the warp
        P = np.array([I] * ns)         # scanned transfers (prefix / suffix)
        for g in range(nw):
            ss = list(range(g * spw, g * spw + spw))[::order]
            prev, Pp = np.zeros(3), I
            for s in ss:
                S[s] = val[s] + T[s] @ prev
                P[s] = T[s] @ Pp
                prev, Pp = S[s], P[s]
        agg = np.array([S[(g * spw + spw - 1) if order > 0 else g * spw] for g in range(nw)])
        Wg = np.array([P[(g * spw + spw - 1) if order > 0 else g * spw] for g in range(nw)])

        def prod(g_from, g_to):        # transfers of the warps strictly between, nearest last
            out = I
            rng_ = range(g_from + order, g_to, order)
            for k in rng_:
                out = Wg[k] @ out
            return out

        cta = [list(range(rw * c, rw * c + rw))[::order] for c in range(ncta)]
        AGG = [sum(prod(k, c_[-1] + order) @ agg[k] for k in c_) for c_ in cta]
        Tc = [prod(c_[0] - order, c_[-1] + order) for c_ in cta]
        cin = np.zeros((nw, 3))
        for g in range(nw):
            c = g // rw
            own = [k for k in cta[c] if (k - g) * order < 0]
            cin[g] = sum((prod(k, g) @ agg[k] for k in own), np.zeros(3))
            K = prod(cta[c][0] - order, g)
            others = range(c - 1, -1, -1) if order > 0 else range(c + 1, ncta)
            for cp in others:
                Psi = I
                for k in range(cp + order, c, order):
                    Psi = Tc[k] @ Psi
                cin[g] += K @ Psi @ AGG[cp]
        carry = np.zeros((ns, 3))      # true carry into each segment
        for g in range(nw):
            ss = list(range(g * spw, g * spw + spw))[::order]
            prev = cin[g]
            for s in ss:
                carry[s] = prev
                prev = S[s] + P[s] @ cin[g]
        return carry

    def fwd_local(s):
        v, T = np.zeros(3), I
        for i in segs[s]:
            v, T = z[i] + M[i] @ v, M[i] @ T
        return v, T

    ycarry = direction(fwd_local, +1)
    y = np.zeros_like(r)
    for s, seg in enumerate(segs):
        v = ycarry[s]
        for i in seg:
            v = z[i] + M[i] @ v
            y[i] = v

    def bwd_local(s):
        u, T = np.zeros(3), I
        for i in reversed(segs[s]):
            u, T = y[i] + H[i] @ u, H[i] @ T
        return u, T

    xcarry = direction(bwd_local, -1)
    x = np.zeros_like(r)
    for s, seg in enumerate(segs):
        u = xcarry[s]
        for i in reversed(seg):
            u = y[i] + H[i] @ u
            x[i] = u
    return x


@pytest.mark.parametrize("n,L,spw,rw,ncta", [(13, 1, 3, 2, 3), (40, 3, 3, 2, 3), (30, 2, 2, 2, 4),
                                             (7, 1, 3, 2, 3), (55, 3, 2, 3, 4), (160, 1, 10, 4, 4)])
def test_direct_carry_sums_match_block_thomas(n, L, spw, rw, ncta):
    """The reference-order sweep's carry structure (warp scans, CTA aggregates through products
    of the later warps' transfers, carries as direct sums over the earlier warps and CTAs, both
    directions) gives the block Thomas solution, on lines that fill some or all of the warps and
    CTAs (the last case: ten segments per warp and four warps per CTA, as in the kernel)."""
    a, b, c, r = random_line(n, seed=200 + n + L)
    Bf, cf = factor(a, b, c)
    x_seq = thomas(a, Bf, cf, r)
    x_dir = direct_carries(a, Bf, cf, r, L, spw, rw, ncta)
    assert np.abs(x_dir - x_seq).max() < 1e-12


def sa_pivots_sequential(a, b, c):
    """scatri's pivots (ref/lreltur.f:337-359): c'_0 = c_0 / b_0, c'_i = c_i / (b_i - a_i c'_{i-1})."""
    n = len(b)
    cp = np.empty(n)
    cp[0] = c[0] / b[0]
    for i in range(1, n):
        cp[i] = c[i] / (b[i] - a[i] * cp[i - 1])
    return cp


def sa_pivots_moebius(a, b, c, lanes=32):
    """The same pivots as the warp-per-line kernel forms them: c'_i is a Moebius map of c'_{i-1},
    the 2x2 matrix M_i = [[0, c_i], [-a_i, b_i]] on homogeneous coordinates (a_0 taken as 0, so
    that M_0 gives c_0 / b_0 whatever it is applied to).  Each lane composes its segment's
    matrices, rescaled by powers of two; an inclusive scan composes the segments; a segment's
    entry pivot is the ratio of the second column of the product of the segments before it, and
    the segment reruns the sequential recurrence from there."""
    n = len(b)
    L = -(-n // lanes)

    def scale(T):
        m = np.abs(T).max()
        return T * 2.0 ** (-np.frexp(m)[1]) if m > 0 and np.isfinite(m) else T

    prods = []
    for s in range(lanes):
        T = np.eye(2)
        for i in range(s * L, min(n, s * L + L)):
            T = np.array([[0.0, c[i]], [-(a[i] if i else 0.0), b[i]]]) @ T
        prods.append(scale(T))
    scan, P = [], np.eye(2)
    for T in prods:  # later segments on the left
        P = scale(T @ P)
        scan.append(P)
    cp = np.empty(n)
    for s in range(lanes):
        beg = s * L
        if beg >= n:
            break
        prev = 0.0 if s == 0 else scan[s - 1][0, 1] / scan[s - 1][1, 1]
        for i in range(beg, min(n, beg + L)):
            prev = c[i] / b[i] if i == 0 else c[i] / (b[i] - a[i] * prev)
            cp[i] = prev
    return cp


@pytest.mark.parametrize("n", [17, 121, 481, 1921])
def test_sa_pivots_by_segment_products_match_the_recurrence(n):
    """The SA line pivots of the warp-per-line factorisation (segment products of the pivot
    recurrence, scanned) equal scatri's sequential recurrence to rounding on diagonally dominant
    lines, including lines far longer than a warp has lanes (the products are rescaled, so
    they neither overflow nor underflow)."""
    rng = np.random.default_rng(n)
    a = -rng.uniform(0.1, 1.0, n)
    c = -rng.uniform(0.1, 1.0, n)
    b = np.abs(a) + np.abs(c) + rng.uniform(0.05, 1.0, n)
    seq = sa_pivots_sequential(a, b, c)
    scan = sa_pivots_moebius(a, b, c)
    assert np.max(np.abs(scan - seq) / np.abs(seq)) < 1e-13


def test_head_point_plan():
    """The plan of the CUDA sweep: a line of n points over 640 segments takes L = ceil(n / 640)
    points per segment, or, when one point fewer needs a smaller L (2 to 4), a head point and
    L = ceil((n - 1) / 640)."""
    def plan(n, cap=640):
        L = -(-n // cap)
        L1 = -(-(n - 1) // cap)
        H = 1 if 2 <= L1 <= 4 and L1 < L else 0
        if H:
            L = L1
        return L, H, -(-(n - H) // L)
    assert plan(481) == (1, 0, 481)
    assert plan(641) == (2, 0, 321)
    assert plan(721) == (2, 0, 361)
    assert plan(1281) == (2, 1, 640)
    assert plan(1921) == (3, 1, 640)
    assert plan(2001) == (4, 0, 501)
    assert plan(2561) == (4, 1, 640)
    for n in range(2, 5121):
        L, H, S = plan(n)
        assert S <= 640 and H + (S - 1) * L < n <= H + S * L
