"""TEST INFRASTRUCTURE ONLY: the benchmark cases built without the product.

The reference ships no grids or input decks, so every case of the tests and
of the benchmark is a seeded algebraic NACA 4-digit C-mesh with a
single-C-mesh &bcinp table.  The product library builds the same inputs
(ot2d_mesh_naca4_cmesh, ot2d_cmesh_bc_table); this module restates them with
numpy and Python's libm calls so that the CPU legs of the benchmark (the
reference arm and the cpu_baseline) never load the product library: with the
oracle's read_inputs (setup.f:876-1268) they give the oracle everything a
solve needs.  tests/test_cpu.py pins the two generators against each other.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this.
"""
import math

import numpy as np


def bc_table(inp, jtail):
    """The five &bcinp entries of a single C-mesh (setup.f:914-931 reads
    them from bc.inp): wall 5 on k = 1 between the trailing-edge vertices,
    wake cut 51 on the lower run of k = 1 (bcwake mirrors it, bc.f:1516),
    and the characteristic far field 47 on k = kmax, j = 1 and j = jmax."""
    jmax, kmax = inp.jmax, inp.kmax
    rows = ((5, 2, jtail, jmax - jtail + 1, 1, 1),
            (51, 2, 1, jtail, 1, 1),
            (47, -2, 1, jmax, kmax, kmax),
            (47, 1, 1, 1, 1, kmax),
            (47, -1, jmax, jmax, 1, kmax))
    inp.nbc = len(rows)
    for i, (t, d, js, je, ks, ke) in enumerate(rows):
        inp.ibtyp[i], inp.ibdir[i], inp.jbcs[i], inp.jbce[i], inp.kbcs[i], inp.kbce[i] = t, d, js, je, ks, ke
    return inp


def _naca4(m, p, t, x):
    """Camber line, its slope and the half thickness of a NACA 4-digit
    section at chord station x (the published NACA 4-digit formulas)."""
    yt = 5.0 * t * (0.2969 * math.sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x
                    - 0.1036 * x * x * x * x)
    if m <= 0.0 or p <= 0.0:
        return 0.0, 0.0, yt
    if x < p:
        return m / (p * p) * (2 * p * x - x * x), 2 * m / (p * p) * (p - x), yt
    return (m / ((1 - p) * (1 - p)) * ((1 - 2 * p) + 2 * p * x - x * x), 2 * m / ((1 - p) * (1 - p)) * (p - x), yt)


def _geometric_ratio(a, n, length):
    """Ratio of the geometric series of n steps from a that sums to length
    (bisection)."""
    if a * n >= length:
        return 1.0
    lo, hi = 1.0 + 1e-12, 4.0
    for _ in range(200):
        r = 0.5 * (lo + hi)
        if a * (math.pow(r, n) - 1.0) / (r - 1.0) > length:
            hi = r
        else:
            lo = r
    return 0.5 * (lo + hi)


def naca4_cmesh(jmax, kmax, n_wake, m=0.0, p=0.0, t=0.12, ds_wall=1e-3, r_far=20.0):
    """Vertices xv, yv as (kmax, jmax) arrays (C order == Fortran (jmax,kmax)).

    j runs clockwise: lower wake from the outflow to the trailing edge, lower
    surface to the leading edge, upper surface, upper wake; k from the wall
    or the cut to the far field.  Cosine-clustered surface, geometric wake and
    wall-normal distributions (first wall spacing ds_wall, far field at r_far
    chords), and lines that blend the smoothed wall normal into the straight
    ray to the outer C boundary with cubic Hermite functions."""
    nsurf = jmax - 2 * n_wake
    if jmax < 9 or kmax < 5 or n_wake < 2 or nsurf < 5 or nsurf % 2 == 0:
        raise ValueError("bad C-mesh sizes")
    half = (nsurf - 1) // 2
    pi = 4.0 * math.atan(1.0)
    bx, by = np.zeros(jmax), np.zeros(jmax)
    for i in range(nsurf):
        lower = i < half
        phi = (half - i) / half if lower else (i - half) / half
        x = 0.5 * (1.0 - math.cos(pi * phi))
        yc, dyc, yt = _naca4(m, p, t, x)
        th = math.atan(dyc)
        j = n_wake + i
        if lower:
            bx[j], by[j] = x + yt * math.sin(th), yc - yt * math.cos(th)
        else:
            bx[j], by[j] = x - yt * math.sin(th), yc + yt * math.cos(th)
        if i in (0, nsurf - 1):
            bx[j], by[j] = 1.0, 0.0
        if i == half:
            bx[j], by[j] = 0.0, 0.0
    # wake on y = 0, geometric from the trailing edge, rescaled to r_far
    ds_te = math.hypot(bx[n_wake + 1] - bx[n_wake], by[n_wake + 1] - by[n_wake])
    rw = _geometric_ratio(ds_te, n_wake, r_far)
    wx = [1.0]
    xw, step = 1.0, ds_te
    for _ in range(n_wake):
        xw += step
        step *= rw
        wx.append(xw)
    scale = r_far / (wx[n_wake] - 1.0)
    for i in range(1, n_wake + 1):
        w = 1.0 + (wx[i] - 1.0) * scale
        bx[n_wake - i], by[n_wake - i] = w, 0.0
        bx[jmax - n_wake - 1 + i], by[jmax - n_wake - 1 + i] = w, 0.0
    # outward wall normals from central differences of the surface
    nx, ny = np.zeros(jmax), np.zeros(jmax)
    for j in range(n_wake, jmax - n_wake):
        if j == n_wake:
            tx, ty = bx[j + 1] - bx[j], by[j + 1] - by[j]
        elif j == jmax - n_wake - 1:
            tx, ty = bx[j] - bx[j - 1], by[j] - by[j - 1]
        else:
            tx, ty = bx[j + 1] - bx[j - 1], by[j + 1] - by[j - 1]
        ln = math.hypot(tx, ty)
        nx[j], ny[j] = -ty / ln, tx / ln
    # 1-2-1 smoothing of the normals with the ends held (4 nsurf passes)
    lo, hi = n_wake + 1, jmax - n_wake - 1
    for _ in range(4 * nsurf):
        tx = 0.25 * nx[lo - 1:hi - 1] + 0.5 * nx[lo:hi] + 0.25 * nx[lo + 1:hi + 1]
        ty = 0.25 * ny[lo - 1:hi - 1] + 0.5 * ny[lo:hi] + 0.25 * ny[lo + 1:hi + 1]
        ln = np.hypot(tx, ty)
        nx[lo:hi], ny[lo:hi] = tx / ln, ty / ln
    nx[:n_wake], ny[:n_wake] = nx[n_wake], ny[n_wake]
    nx[jmax - n_wake:], ny[jmax - n_wake:] = nx[jmax - n_wake - 1], ny[jmax - n_wake - 1]
    # directions turn monotonically from the leading edge to both outflow ends
    jle0 = n_wake + half
    amax = -1e30
    for j in range(jle0, -1, -1):
        a = math.atan2(ny[j], nx[j])
        if a > 0.5 * pi:
            a -= 2.0 * pi
        a = max(a, amax)
        amax = a
        nx[j], ny[j] = math.cos(a), math.sin(a)
    amin = 1e30
    for j in range(jle0, jmax):
        a = math.atan2(ny[j], nx[j])
        if a < -0.5 * pi:
            a += 2.0 * pi
        a = min(a, amin)
        amin = a
        nx[j], ny[j] = math.cos(a), math.sin(a)
    # outer boundary: y = -/+ r_far downstream, a semicircle about the TE
    ox, oy = np.zeros(jmax), np.zeros(jmax)
    for j in range(jmax):
        if j < n_wake:
            ox[j], oy[j] = bx[j], -r_far
        elif j > jmax - n_wake - 1:
            ox[j], oy[j] = bx[j], r_far
        else:
            ang = -0.5 * pi - pi * ((j - n_wake) / (nsurf - 1))
            ox[j], oy[j] = 1.0 + r_far * math.cos(ang), r_far * math.sin(ang)
    # geometric wall-normal coordinate eta in [0, 1]
    K = kmax - 1
    a = ds_wall / r_far
    rk = _geometric_ratio(a, K, 1.0)
    eta = [0.0]
    st, acc = a, 0.0
    for _ in range(K):
        acc += st
        st *= rk
        eta.append(acc)
    eta = np.array([0.0] + [e / eta[K] for e in eta[1:]])
    dx, dy = ox - bx, oy - by
    D = np.hypot(dx, dy)
    t0x, t0y = nx * D, ny * D
    e = eta[:, None]
    e2 = e * e
    e3 = e2 * e
    h0, h1, h2, h3 = 2 * e3 - 3 * e2 + 1, -2 * e3 + 3 * e2, e3 - 2 * e2 + e, e3 - e2
    xv = h0 * bx + h1 * ox + h2 * t0x + h3 * dx
    yv = h0 * by + h1 * oy + h2 * t0y + h3 * dy
    # the two wake runs share the cut exactly
    xv[0, jmax - 1 - np.arange(n_wake + 1)] = xv[0, :n_wake + 1]
    yv[0, jmax - 1 - np.arange(n_wake + 1)] = yv[0, :n_wake + 1]
    if m <= 0.0 or p <= 0.0:
        # a symmetric section gets an exactly mirror-symmetric grid
        mid = (jmax - 1) // 2
        xv[:, jmax - 1 - np.arange(mid)] = xv[:, :mid]
        yv[:, jmax - 1 - np.arange(mid)] = -yv[:, :mid]
        yv[:, mid] = 0.0
    return np.ascontiguousarray(xv), np.ascontiguousarray(yv)


def wall_spacing(kmax, r_far=20.0, ratio=1.2, floor=1e-6):
    """First-cell wall spacing whose geometric stretching at `ratio` reaches
    the far field over kmax points, but not below `floor` chords."""
    return max(floor, r_far * (ratio - 1.0) / (ratio ** (kmax - 1) - 1.0))


def c2_inputs(jmax=513, kmax=129, fsmach=0.15, alfa=10.0, rey=6e6, naca=(0.0, 0.0, 0.12), ds_wall=1e-6):
    """Namelist + grid of the RANS-SA case: NACA C-mesh, MUSCL (irhsy -3,
    ilim 1) + Roe, LU-SGS at local CFL 50, nu_tilde_inf = 3 nu_inf.  Returns
    (inputs, xv, yv); the oracle's read_inputs turns the inputs into the
    module state."""
    from turns2d_urans_git_gb300.abi import default_inputs   # ctypes structs only
    n_wake = (jmax - 1) // 8
    inp = default_inputs(jmax=jmax, kmax=kmax, invisc=0, lamin=0, iturb=1, irhsy=-3, ilim=1, ilhs=1,
                         iconstant_cfl=1, dt=50.0, fsmach=fsmach, alfa=alfa, rey=rey, vnuinf=3.0)
    bc_table(inp, n_wake + 1)
    xv, yv = naca4_cmesh(jmax, kmax, n_wake, naca[0], naca[1], naca[2], ds_wall, 20.0)
    return inp, xv, yv
