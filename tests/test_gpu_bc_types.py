"""Boundary-condition types beyond the C-mesh table (bc.f:2-85, rbc
bc.f:88-177), on O-meshes whose &bcinp tables use them:

  3   inviscid wall (bcwall, bc.f:1669-1801)        k = 1
  4   viscous wall (bcwall)                         k = 1
  22  periodic, overlapping planes (bc.f:180-357)   j = 1 and j = jmax of a closed O-mesh
  11  symmetry (bcsym, bc.f:2096-2157)              j = 1 and j = jmax of a half O-mesh
  46  freestream (bcout_inf, bc.f:360-407)          k = kmax
  10  extrapolation (bcextp, bc.f:1962-2026)        k = kmax

Each table goes through one drop-in bc and rbc call on a perturbed state
and a 30-iteration FP64 solve of the batched solver, both against the
oracle at 1e-12 (1e-10 for the SA case: its real powers go through two
libms)."""
import ctypes as C

import numpy as np
import pytest

from tests import oracle_binding as ob
from tests.helpers import relerr
from turns2d_urans_git_gb300 import api
from turns2d_urans_git_gb300 import routines as rt
from turns2d_urans_git_gb300.abi import OT2D_FP64, default_inputs

pytestmark = pytest.mark.gpu


def omesh(jmax, kmax, ds, r_far=20.0, half=False):
    """Vertices of an O-mesh around a circle of diameter 1 (centre (0.5, 0)):
    j runs clockwise from the downstream axis (the full circle: first and
    last vertex lines coincide; half: the upper half, from the upstream axis
    to the downstream one), k outwards with geometric spacing from ds."""
    K = kmax - 1
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        r = 0.5 * (lo + hi)
        if ds * (r ** K - 1.0) / (r - 1.0) > r_far:
            hi = r
        else:
            lo = r
    rad = 0.5 + np.concatenate([[0.0], np.cumsum(ds * r ** np.arange(K))])
    if half:
        th = np.pi * (1.0 - np.arange(jmax) / (jmax - 1))       # pi -> 0, clockwise over the top
    else:
        th = -2.0 * np.pi * np.arange(jmax) / (jmax - 1)        # 0 -> -2 pi, clockwise
    xv = 0.5 + rad[:, None] * np.cos(th)[None, :]
    yv = rad[:, None] * np.sin(th)[None, :]
    if not half:
        xv[:, -1], yv[:, -1] = xv[:, 0], yv[:, 0]              # the seam: coincident vertex lines
    else:
        yv[:, 0] = 0.0
        yv[:, -1] = 0.0
    return np.ascontiguousarray(xv), np.ascontiguousarray(yv)


def _table(inp, rows):
    inp.nbc = len(rows)
    for i, (t, d, js, je, ks, ke) in enumerate(rows):
        inp.ibtyp[i], inp.ibdir[i], inp.jbcs[i], inp.jbce[i], inp.kbcs[i], inp.kbce[i] = t, d, js, je, ks, ke
    return inp


def _variant(kind):
    if kind == "periodic_wall3_freestream":
        jm, km = 97, 33
        inp = default_inputs(jmax=jm, kmax=km, invisc=1, lamin=1, irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1,
                             dt=5.0, fsmach=0.3, alfa=2.0)
        _table(inp, [(3, 2, 1, jm, 1, 1), (22, 1, 1, 1, 1, km), (22, -1, jm, jm, 1, km), (46, -2, 1, jm, km, km)])
        xv, yv = omesh(jm, km, 2e-3)
    elif kind == "periodic_wall4_extrapolation":
        jm, km = 97, 41
        inp = default_inputs(jmax=jm, kmax=km, invisc=0, lamin=0, iturb=1, irhsy=-3, ilim=1, ilhs=1,
                             iconstant_cfl=1, dt=10.0, fsmach=0.3, alfa=2.0, rey=1e5, vnuinf=3.0)
        _table(inp, [(4, 2, 1, jm, 1, 1), (22, 1, 1, 1, 1, km), (22, -1, jm, jm, 1, km), (10, -2, 1, jm, km, km)])
        xv, yv = omesh(jm, km, 1e-3)
    else:  # symmetry_wall3_freestream
        jm, km = 65, 33
        inp = default_inputs(jmax=jm, kmax=km, invisc=1, lamin=1, irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1,
                             dt=5.0, fsmach=0.3, alfa=0.0)
        _table(inp, [(3, 2, 1, jm, 1, 1), (11, 1, 1, 1, 1, km), (11, -1, jm, jm, 1, km), (46, -2, 1, jm, km, km)])
        xv, yv = omesh(jm, km, 2e-3, half=True)
    return inp, xv, yv


KINDS = ["periodic_wall3_freestream", "periodic_wall4_extrapolation", "symmetry_wall3_freestream"]


def _arrays(p, xv, yv, seed):
    """Geometry and a perturbed physical state set up by the oracle
    (find_cellcenter, metfv, qzero, qdivj)."""
    n2 = p.jd * p.kd
    z = lambda: np.zeros(n2)
    a = dict(x=z(), y=z(), xx=z(), xy=z(), yx=z(), yy=z(), ug=z(), vg=z(), bt=z(), q=np.zeros(n2 * p.nq))
    L, pp = ob.lib(), C.byref(p)
    xvf, yvf = np.ascontiguousarray(xv.ravel()), np.ascontiguousarray(yv.ravel())
    L.oro_find_cellcenter(pp, ob.ptr(a["x"]), ob.ptr(a["y"]), ob.ptr(xvf), ob.ptr(yvf))
    assert L.oro_metfv(pp, ob.ptr(a["q"]), ob.ptr(xvf), ob.ptr(yvf), ob.ptr(a["xx"]), ob.ptr(a["xy"]),
                       ob.ptr(a["yx"]), ob.ptr(a["yy"])) == 0
    L.oro_qzero(pp, ob.ptr(a["q"]))
    L.oro_qdivj(pp, ob.ptr(a["q"]))
    rng = np.random.default_rng(seed)
    q = a["q"].reshape(p.nq, n2)
    J = q[p.nq - 1]
    rho = q[0] * J * (1.0 + 0.02 * rng.uniform(-1, 1, n2))
    u = q[1] / q[0] + 0.02 * rng.uniform(-1, 1, n2)
    v = q[2] / q[0] + 0.02 * rng.uniform(-1, 1, n2)
    pres = p.pinf * (1.0 + 0.02 * rng.uniform(-1, 1, n2))
    q[0], q[1], q[2] = rho / J, rho * u / J, rho * v / J
    q[3] = (pres / p.gm1 + 0.5 * rho * (u * u + v * v)) / J
    if not p.lamin:
        q[4] = p.vnuinf * (1.0 + 50.0 * rng.uniform(0, 1, n2))
    return a


@pytest.mark.parametrize("kind", KINDS)
def test_bc_and_rbc_dropin_match_oracle(kind):
    inp, xv, yv = _variant(kind)
    p = ob.read_inputs(inp)
    assert bytes(p) == bytes(api.params_from_inputs(inp))
    p.istep0 = 10                                          # inside the 30-step wall ramp
    a = _arrays(p, xv, yv, seed=3)
    n2 = p.jd * p.kd
    qo, qg = a["q"].copy(), a["q"].copy()
    L = ob.lib()
    L.oro_bc(C.byref(p), ob.ptr(qo), ob.ptr(a["xx"]), ob.ptr(a["xy"]), ob.ptr(a["yx"]), ob.ptr(a["yy"]),
             ob.ptr(a["ug"]), ob.ptr(a["vg"]), ob.ptr(a["bt"]))
    rt.set_params(p)
    rt.bc(qg, a["x"], a["y"], a["xx"], a["xy"], a["yx"], a["yy"], a["ug"], a["vg"], 1, p.jd, p.kd, a["bt"])
    assert not np.array_equal(qo, a["q"])                  # the BCs changed the halo
    assert relerr(qg, qo) <= 1e-12
    so = np.random.default_rng(9).uniform(-1, 1, n2 * p.nv) * 1e-4
    sg = so.copy()
    L.oro_rbc(C.byref(p), ob.ptr(qo), ob.ptr(so))
    rt.rbc(qo.copy(), sg, a["x"], a["y"], a["xx"], a["xy"], a["yx"], a["yy"], a["ug"], a["vg"], 1, p.jd, p.kd,
           a["bt"])
    assert relerr(sg, so) <= 1e-12


@pytest.mark.parametrize("kind", KINDS)
def test_solver_with_bc_types_matches_oracle(kind):
    inp, xv, yv = _variant(kind)
    p = api.params_from_inputs(inp)
    nsteps = 30
    n, hist, forces, q_o = ob.solve(p, xv.ravel(), yv.ravel(), nsteps)
    assert n == nsteps
    sv = api.Solver(OT2D_FP64, check_every=nsteps, keep_q=True)
    iid = sv.add(p, xv, yv, orders=0.0, max_iters=nsteps)
    sv.iterate(nsteps)
    sv.sync()
    r = sv.result(iid)
    q = sv.get_q(iid, p)
    sv.close()
    tol = 1e-10 if not p.lamin else 1e-12
    assert r.status == 0 and r.iterations == nsteps
    assert abs(r.rsum_last - hist[-1, 0]) <= tol * hist[-1, 0]
    assert relerr(q, q_o) <= tol
    for g, o in ((r.cl, forces[0][0]), (r.cd, forces[0][1]), (r.cm, forces[0][2])):
        assert abs(g - o) <= tol * max(abs(o), 1e-3)
