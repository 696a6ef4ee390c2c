"""GPU parity of Turkel's low-Mach preconditioning (iprecon, Mp) against the
CPU FP64 oracle, through the C-ABI: the drop-in rhsup with roetrklflx
(eulerrhs.f:450-625), rhslom (sources.f:97-148), preilu2d (lhs.f:2-467) and
arc2d_precon (lhs.f:1060-1330), and the batched solver / drop-in step with
them in the iteration (step.f:121-123, :154-180; time.f:30-35, :62-66).

bt comes from a dual-time time step (idual = 1), so bSq = Mp**2/(bt -
Mp**2 (bt-1)) differs from cell to cell.

Tolerance: 1e-12 relative for the FP64 path, as for every other FP64
routine (the kernels keep the reference's operation order without fused
multiply-adds); the FP32-mixed solver is compared with FP64 on its forces.
"""
import ctypes as C

import numpy as np
import pytest

from tests import oracle_binding as ob
from tests.helpers import Case, relerr
from turns2d_urans_git_gb300 import api, routines as rt
from turns2d_urans_git_gb300.abi import OT2D_FP64, OT2D_FP32_MIXED

pytestmark = pytest.mark.gpu
TOL = 1e-12
MP = 0.3


def _o(c):
    return C.byref(c.p)


def _pcase(viscous=False, seed=31, ilim=1, irhsy=-3, fsmach=0.2):
    """A perturbed low-Mach state with preconditioning on and the dual-time
    step's bt (time.f:57-72) in c.bt."""
    c = Case(viscous=viscous, seed=seed, ilim=ilim, irhsy=irhsy, fsmach=fsmach)
    c.p.iprecon, c.p.Mp, c.p.idual, c.p.idual_turb = 1, MP, 1, 1
    ob.lib().oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                           ob.ptr(c.vg), ob.ptr(c.tscale), ob.ptr(c.bt), ob.ptr(c.iblank))
    assert np.ptp(c.bt[c.bt > 0]) > 0   # bt varies: bSq is cell dependent
    return c


def test_time_step_precon():
    """time.f:62-66: the preconditioned dual-time tscale (iconstant_cfl 0)."""
    for visc in (False, True):
        c = _pcase(viscous=visc, seed=30)
        c.p.iconstant_cfl = 0
        ts_o, bt_o = np.zeros(c.n2), np.zeros(c.n2)
        ob.lib().oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy),
                               ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(ts_o), ob.ptr(bt_o), ob.ptr(c.iblank))
        rt.set_params(c.p)
        ts, bt = np.zeros(c.n2), np.zeros(c.n2)
        rt.time_step(c.q, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, ts, bt, c.iblank, c.jd, c.kd)
        assert relerr(ts, ts_o) <= TOL and relerr(bt, bt_o) <= TOL


@pytest.mark.parametrize("ilim,irhsy", [(0, -3), (1, -3), (4, -3), (1, -1)])
def test_rhsup_turkel(ilim, irhsy):
    c = _pcase(seed=32, ilim=ilim, irhsy=irhsy)
    so = np.random.default_rng(9).uniform(-1, 1, c.n2 * c.p.nv) * 1e-3
    s = so.copy()
    ob.lib().oro_rhsup(_o(c), ob.ptr(c.q), ob.ptr(so), ob.ptr(c.xv), ob.ptr(c.yv), ob.ptr(c.iblank), ob.ptr(c.ugv),
                       ob.ptr(c.vgv))
    rt.set_params(c.p)
    rt.rhsup(c.q, s, c.xx, c.xy, c.yx, c.yy, c.x, c.y, c.xv, c.yv, c.xv, c.yv, c.xv, c.yv, c.iblank, c.ugv, c.vgv,
             c.jd, c.kd, 1, 1, c.bt)
    assert relerr(s, so) <= TOL
    # the preconditioned flux really differs from roeflx
    c.p.iprecon = 0
    s0 = np.random.default_rng(9).uniform(-1, 1, c.n2 * c.p.nv) * 1e-3
    ob.lib().oro_rhsup(_o(c), ob.ptr(c.q), ob.ptr(s0), ob.ptr(c.xv), ob.ptr(c.yv), ob.ptr(c.iblank), ob.ptr(c.ugv),
                       ob.ptr(c.vgv))
    assert relerr(s0, so) > 1e-6


def test_rhslom():
    c = _pcase(seed=33)
    so = np.random.default_rng(4).uniform(-1, 1, c.n2 * c.p.nv) * 1e-3
    s = so.copy()
    ob.lib().oro_rhslom(_o(c), ob.ptr(c.q), ob.ptr(so), ob.ptr(c.bt))
    rt.set_params(c.p)
    p = c.p
    rt.rhslom(c.q, s, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.bt)
    assert not np.array_equal(s, np.random.default_rng(4).uniform(-1, 1, c.n2 * c.p.nv) * 1e-3)
    assert relerr(s, so) <= TOL


@pytest.mark.parametrize("visc", [False, True])
def test_preilu2d(visc):
    c = _pcase(viscous=visc, seed=34)
    L = ob.lib()
    so = np.random.default_rng(3).uniform(-1, 1, c.n2 * c.p.nv) * 1e-4
    s, qo, q = so.copy(), c.q.copy(), c.q.copy()
    L.oro_preilu2d(_o(c), ob.ptr(qo), ob.ptr(so), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy),
                   ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(c.turmu), ob.ptr(c.tscale), ob.ptr(c.bt))
    rt.set_params(c.p)
    p = c.p
    rt.preilu2d(q, s, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.turmu,
                c.tscale, c.bt)
    assert relerr(s, so) <= TOL
    assert relerr(q, qo) <= TOL
    # ilu2d on the same input stays the plain operator (the call chooses,
    # not params iprecon)
    s2, q2 = np.random.default_rng(3).uniform(-1, 1, c.n2 * c.p.nv) * 1e-4, c.q.copy()
    so2, qo2 = s2.copy(), c.q.copy()
    L.oro_ilu2d(_o(c), ob.ptr(qo2), ob.ptr(so2), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy),
                ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(c.turmu), ob.ptr(c.tscale))
    rt.ilu2d(q2, s2, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.turmu,
             c.tscale)
    assert relerr(s2, so2) <= TOL
    assert relerr(s2, s) > 1e-6


@pytest.mark.parametrize("visc,ilhs", [(False, 2), (True, 2), (True, 3)])
def test_arc2d_precon(visc, ilhs):
    c = _pcase(viscous=visc, seed=35)
    c.p.ilhs = ilhs
    L = ob.lib()
    so = np.random.default_rng(23).uniform(-1, 1, c.n2 * c.p.nv) * 1e-4
    s, qo, q = so.copy(), c.q.copy(), c.q.copy()
    L.oro_arc2d_precon(_o(c), ob.ptr(qo), ob.ptr(so), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy),
                       ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(c.turmu), ob.ptr(c.iblank), ob.ptr(c.tscale), ob.ptr(c.bt))
    rt.set_params(c.p)
    p = c.p
    rt.arc2d_precon(q, s, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.turmu,
                    c.iblank, c.tscale, c.bt)
    assert relerr(s[:4 * c.n2], so[:4 * c.n2]) <= TOL
    assert relerr(q, qo) <= TOL
    # arc2d on the same input stays the plain operator
    s2 = np.random.default_rng(23).uniform(-1, 1, c.n2 * c.p.nv) * 1e-4
    rt.arc2d(c.q.copy(), s2, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg,
             c.turmu, c.iblank, c.tscale, c.bt)
    assert relerr(s2[:4 * c.n2], s[:4 * c.n2]) > 1e-6


def _precon_case(kind):
    if kind == "euler":
        _, prm, xv, yv = api.cmesh_case(97, 25, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=1, lamin=1, irhsy=-3,
                                        ilim=1, ilhs=1, iconstant_cfl=1, dt=2.0, fsmach=0.1, alfa=2.0)
    elif kind == "euler_weno":
        _, prm, xv, yv = api.cmesh_case(97, 25, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=1, lamin=1, irhsy=-3,
                                        ilim=4, ilhs=1, iconstant_cfl=0, dt=2.0, fsmach=0.1, alfa=2.0)
    elif kind == "euler_adi":
        _, prm, xv, yv = api.cmesh_case(97, 25, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=1, lamin=1, irhsy=-3,
                                        ilim=1, ilhs=2, iconstant_cfl=1, dt=2.0, fsmach=0.1, alfa=2.0)
    elif kind == "sa_adi_up":
        _, prm, xv, yv = api.cmesh_case(97, 33, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=1,
                                        irhsy=-3, ilim=1, ilhs=3, iconstant_cfl=1, dt=5.0, fsmach=0.15, alfa=3.0,
                                        rey=1e6, vnuinf=3.0)
    else:
        _, prm, xv, yv = api.cmesh_case(97, 33, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=1,
                                        irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1, dt=5.0, fsmach=0.15, alfa=3.0,
                                        rey=1e6, vnuinf=3.0)
    prm.iprecon, prm.Mp = 1, MP
    return prm, xv, yv


@pytest.mark.parametrize("kind", ["euler", "euler_weno", "sa", "euler_adi", "sa_adi_up"])
def test_solver_precon_fp64_matches_oracle(kind):
    """The batched solver with iprecon (roetrklflx, rhslom, preilu2d, the
    dual-time switch of time.f:30-35), FP64, against the oracle driver."""
    prm, xv, yv = _precon_case(kind)
    n_it = 40
    n, hist, forces, q_o = ob.solve(prm, xv.ravel(), yv.ravel(), n_it)
    assert n == n_it
    sv = api.Solver(OT2D_FP64, check_every=n_it, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=n_it)
    sv.iterate(n_it)
    r = sv.result(iid)
    q = sv.get_q(iid, prm)
    sv.close()
    assert r.status == 0 and r.iterations == n_it
    assert relerr(q, q_o) <= TOL
    assert abs(r.rsum_last - hist[-1, 0]) <= 1e-10 * hist[-1, 0]


def test_solver_mixed_batch_precon_and_plain():
    """One batch holding a preconditioned and a plain instance: each equals
    its own oracle solve (the two kernel instantiations split the slices)."""
    prm, xv, yv = _precon_case("euler")
    plain = type(prm).from_buffer_copy(prm)
    plain.iprecon, plain.Mp = 0, 1.0
    n_it = 30
    refs = [ob.solve(p, xv.ravel(), yv.ravel(), n_it)[3] for p in (prm, plain)]
    sv = api.Solver(OT2D_FP64, check_every=n_it, keep_q=True)
    ids = [sv.add(p, xv, yv, orders=0.0, max_iters=n_it) for p in (prm, plain)]
    sv.iterate(n_it)
    for iid, p, q_o in zip(ids, (prm, plain), refs):
        assert sv.result(iid).iterations == n_it
        assert relerr(sv.get_q(iid, p), q_o) <= TOL
    sv.close()


def test_solver_precon_mixed_close_to_fp64():
    prm, xv, yv = _precon_case("euler")
    out = {}
    for prec in (OT2D_FP64, OT2D_FP32_MIXED):
        sv = api.Solver(prec, check_every=100)
        iid = sv.add(prm, xv, yv, orders=0.0, max_iters=200)
        sv.iterate(200)
        out[prec] = sv.result(iid)
        sv.close()
    a, b = out[OT2D_FP32_MIXED], out[OT2D_FP64]
    assert a.status == 0 and a.iterations == 200
    assert abs(a.cl - b.cl) <= 1e-3 and abs(a.cd - b.cd) <= 1e-3


def test_dropin_step_precon_matches_oracle():
    """time_step + step (+ monitor) through the drop-in routines with
    iprecon, as the reference's driver calls them, against the oracle."""
    prm, xv0, yv0 = _precon_case("euler")
    n_it = 12
    n, hist, forces, q_o = ob.solve(prm, xv0.ravel(), yv0.ravel(), n_it)
    p = type(prm).from_buffer_copy(prm)
    p.idual, p.idual_turb = 1, 1   # time.f:30-35, as the first time step sets them
    jd, kd, n2, nvert = p.jd, p.kd, p.jd * p.kd, p.jmax * p.kmax
    xv = np.ascontiguousarray(xv0.ravel(), dtype=np.float64)
    yv = np.ascontiguousarray(yv0.ravel(), dtype=np.float64)
    z = lambda m=1: np.zeros(n2 * m)
    x, y, xx, xy, yx, yy, ug, vg = z(), z(), z(), z(), z(), z(), z(), z()
    turmu, tscale, bt = z(), z(), z()
    q, s = z(p.nq), z(p.nv)
    iblank = np.ones(n2, dtype=np.int32)
    ugv, vgv = np.zeros(nvert), np.zeros(nvert)
    L, pp = ob.lib(), C.byref(p)
    L.oro_find_cellcenter(pp, ob.ptr(x), ob.ptr(y), ob.ptr(xv), ob.ptr(yv))
    assert L.oro_metfv(pp, ob.ptr(q), ob.ptr(xv), ob.ptr(yv), ob.ptr(xx), ob.ptr(xy), ob.ptr(yx), ob.ptr(yy)) == 0
    L.oro_qzero(pp, ob.ptr(q))
    L.oro_qdivj(pp, ob.ptr(q))
    p.istep0 = 0
    for it in range(1, n_it + 1):
        p.istep0 += 1
        p.istep = it
        rt.set_params(p)
        rt.time_step(q, xx, xy, yx, yy, ug, vg, tscale, bt, iblank, jd, kd)
        rt.step(q, None, None, None, s, x, y, xv, yv, iblank, xx, xy, yx, yy, ug, vg, ugv, vgv, None, None, None,
                None, turmu, tscale, bt, np.zeros(1), 1, jd, kd)
        assert rt.monitor(q, jd, kd) == 0
    assert relerr(q, q_o) <= TOL
