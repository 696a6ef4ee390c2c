"""GPU parity of the time-accurate path (iunst = 1, motiontype = 1): a
pitching NACA 0012 advanced by dual time stepping -- per physical step the
grid rotation, metrics, face speeds and wall distances on the device
(motion.f pitch, setup.f metfv, eulerrhs.f swept-area face speeds,
samodel2d.f dist), stqol, then itnmax Newton iterations with the physical-time
term of newton -- through the batched solver, against the oracle driver
running the same Turns_overset.f loop.

Tolerance: 1e-12 relative on the state for Euler and SA (the FP64 path keeps
the reference's operation order, including the geometry); 1e-10 for SST, as
in the steady SST test (pow / exp of its source terms may differ by an ulp).
"""
import numpy as np
import pytest

from tests import oracle_binding as ob
from tests.helpers import relerr
from turns2d_urans_git_gb300 import api
from turns2d_urans_git_gb300.abi import OT2D_FP64, OT2D_FP32_MIXED

pytestmark = pytest.mark.gpu

CASES = {
    # name: (config_pitching kwargs, physical steps, state tolerance)
    "euler_ntac2": (dict(jmax=97, kmax=25, ntac=2, itnmax=4, dt=0.1, rf=0.5, angmax=2.0), 8, 1e-12),
    "euler_ntac1": (dict(jmax=97, kmax=25, ntac=1, itnmax=3, dt=0.1, rf=0.5, angmax=2.0), 6, 1e-12),
    "euler_ntac3": (dict(jmax=97, kmax=25, ntac=3, itnmax=3, dt=0.1, rf=0.5, angmax=2.0), 6, 1e-12),
    "sa_ntac2": (dict(jmax=97, kmax=33, viscous=True, iturb=1, ntac=2, itnmax=3, dt=0.1, rf=0.5, angmax=2.0), 5,
                 1e-12),
    "sst_ntac2": (dict(jmax=97, kmax=33, viscous=True, iturb=2, ntac=2, itnmax=3, dt=0.1, rf=0.5, angmax=2.0), 5,
                  1e-10),
}


@pytest.mark.parametrize("kind", sorted(CASES))
def test_solver_pitching_fp64_matches_oracle(kind):
    kw, nsteps, tol = CASES[kind]
    _, prm, xv, yv = api.config_pitching(**kw)
    n, hist, forces, q_o = ob.solve(prm, xv.ravel(), yv.ravel(), nsteps)
    assert n == nsteps
    # a status-check interval that does not divide the iteration count: the
    # instance still stops after exactly nsteps physical steps
    sv = api.Solver(OT2D_FP64, check_every=7, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=nsteps)
    sv.iterate(nsteps * prm.itnmax + 20)
    assert sv.live() == 0
    r = sv.result(iid)
    q = sv.get_q(iid, prm)
    sv.close()
    assert r.status == 0 and r.iterations == nsteps, (r.status, r.iterations)
    assert relerr(q, q_o) <= tol
    assert abs(r.rsum_last - hist[-1, 0]) <= 1e-9 * hist[-1, 0]
    f = forces[0]
    for a, b in ((r.cl, f[0]), (r.cd, f[1]), (r.cm, f[2])):
        assert abs(a - b) <= 100 * tol * max(abs(b), 1e-3)


def test_solver_pitching_mixed_close_to_fp64():
    """The FP32-mixed path on the same pitching Euler case: forces within
    1e-4 of FP64 after 8 physical steps (the f32 residual has no freestream
    correction on a moving grid)."""
    _, prm, xv, yv = api.config_pitching(jmax=97, kmax=25, ntac=2, itnmax=4, dt=0.1, rf=0.5, angmax=2.0)
    out = {}
    for prec in (OT2D_FP64, OT2D_FP32_MIXED):
        sv = api.Solver(prec, check_every=100)
        iid = sv.add(prm, xv, yv, orders=0.0, max_iters=8)
        sv.iterate(8 * prm.itnmax)
        assert sv.live() == 0
        out[prec] = sv.result(iid)
        sv.close()
    a, b = out[OT2D_FP32_MIXED], out[OT2D_FP64]
    assert a.status == 0 and a.iterations == 8
    assert abs(a.cl - b.cl) <= 1e-4 and abs(a.cd - b.cd) <= 1e-4


def test_steady_instance_stops_exactly_at_its_cap():
    """A steady instance whose cap is not a multiple of the status-check
    interval runs exactly max_iters iterations."""
    _, prm, xv, yv = api.config_c1(jmax=65, kmax=25)
    n, hist, forces, q_o = ob.solve(prm, xv.ravel(), yv.ravel(), 30)
    sv = api.Solver(OT2D_FP64, check_every=25, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=30)
    sv.iterate(100)
    r = sv.result(iid)
    q = sv.get_q(iid, prm)
    sv.close()
    assert r.iterations == 30
    assert relerr(q, q_o) <= 1e-12


@pytest.mark.parametrize("kind", ["euler_ntac2", "sa_ntac2"])
def test_dropin_time_loop_matches_oracle(kind):
    """The Turns_overset.f:360-505 loop driven through the drop-in routines,
    as a Fortran driver would call them: per physical step ot2d_pitch,
    ot2d_metfv, ot2d_stqol, then itnmax x (ot2d_time_step, ot2d_step,
    ot2d_monitor); the state equals the oracle driver's."""
    import ctypes as C
    from turns2d_urans_git_gb300 import routines as rt
    kw, nsteps, tol = CASES[kind]
    nsteps = min(nsteps, 4)
    _, prm, xv0, yv0 = api.config_pitching(**kw)
    n, hist, forces, q_o = ob.solve(prm, xv0.ravel(), yv0.ravel(), nsteps)
    assert n == nsteps
    p = type(prm).from_buffer_copy(prm)
    jd, kd, n2, nvert = p.jd, p.kd, p.jd * p.kd, p.jmax * p.kmax
    xv = np.ascontiguousarray(xv0.ravel(), dtype=np.float64)
    yv = np.ascontiguousarray(yv0.ravel(), dtype=np.float64)
    z = lambda m=1: np.zeros(n2 * m)
    x, y, xx, xy, yx, yy, ug, vg = z(), z(), z(), z(), z(), z(), z(), z()
    turmu, tscale, bt = z(), z(), z()
    q, s = z(p.nq), z(p.nv)
    qtn, qtnm1, qnewt = z(p.nv), z(p.nv), z(p.nv)
    iblank = np.ones(n2, dtype=np.int32)
    ugv, vgv = np.zeros(nvert), np.zeros(nvert)
    Ds = np.zeros(1)
    # initia (init.f): centres, metrics, freestream Q/J -- set up by the oracle
    L, pp = ob.lib(), C.byref(p)
    L.oro_find_cellcenter(pp, ob.ptr(x), ob.ptr(y), ob.ptr(xv), ob.ptr(yv))
    assert L.oro_metfv(pp, ob.ptr(q), ob.ptr(xv), ob.ptr(yv), ob.ptr(xx), ob.ptr(xy), ob.ptr(yx), ob.ptr(yy)) == 0
    L.oro_qzero(pp, ob.ptr(q))
    L.oro_qdivj(pp, ob.ptr(q))
    xold, yold, xole, yole = xv.copy(), yv.copy(), xv.copy(), yv.copy()
    p.istep0 = 0
    for istep in range(1, nsteps + 1):
        p.istep0 += 1
        p.istep = istep
        p.totime += p.dt
        rt.set_params(p)
        rt.pitch(x, y, xv, yv, xold, yold, xole, yole, ug, vg, jd, kd)
        rt.metfv(q, x, y, xv, yv, xx, xy, yx, yy, jd, kd)
        if p.itnmax > 1:
            rt.stqol(q, qtn, qtnm1, qnewt, jd, kd)
        for itn in range(1, p.itnmax + 1):
            p.itn = itn
            rt.set_params(p)
            rt.time_step(q, xx, xy, yx, yy, ug, vg, tscale, bt, iblank, jd, kd)
            rt.step(q, qtn, qtnm1, qnewt, s, x, y, xv, yv, iblank, xx, xy, yx, yy, ug, vg, ugv, vgv, xold, yold,
                    xole, yole, turmu, tscale, bt, Ds, 1, jd, kd)
            assert rt.monitor(q, jd, kd) == 0
    assert relerr(q, q_o) <= tol


@pytest.mark.parametrize("visc", [False, True])
def test_step_newton_time_spectral_matches_oracle(visc):
    """step.f with the time-spectral form and Newton sub-iterations (itnmax
    > 1): newtonTS (time.f:213-241) gathers -(q - qnewt)/tscale in ss, which
    is added to s after the norms (step.f:125-131), beside the
    timespectralrhs coupling of the three instances.  Two consecutive
    drop-in steps against the oracle's step."""
    import ctypes as C
    from tests.helpers import Case
    from turns2d_urans_git_gb300 import routines as rt
    ns = 3
    c = Case(viscous=visc, seed=61, perturb=0.01)
    p = type(c.p).from_buffer_copy(c.p)
    p.timespectral, p.nspec, p.itnmax, p.rotf = 1, ns, 2, 0.1
    n2 = c.n2
    rng = np.random.default_rng(62)
    rep = lambda a: np.ascontiguousarray(np.tile(a, ns))
    x, y, xx, xy, yx, yy, ug, vg = (rep(a) for a in (c.x, c.y, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg))
    xv, yv, ugv, vgv = (rep(a) for a in (c.xv, c.yv, c.ugv, c.vgv))
    iblank = rep(c.iblank)
    qc = c.q.reshape(p.nq, n2)
    q = np.concatenate([np.concatenate([qc[n] * (1.0 + 0.003 * i * rng.uniform(-1, 1, n2)) if n < p.nq - 1 else qc[n]
                                        for i in range(ns)]) for n in range(p.nq)])
    qnewt = q[:n2 * ns * p.nv] * (1.0 + 1e-3 * rng.uniform(-1, 1, n2 * ns * p.nv))
    Ds = np.zeros(ns * ns)
    ob.lib().oro_computeTScoefs(ns, ob.ptr(Ds))
    arrs = {}
    for who in ("oracle", "gpu"):
        arrs[who] = dict(q=q.copy(), s=np.zeros(n2 * ns * p.nv), turmu=rep(c.turmu), tscale=np.zeros(n2 * ns),
                         bt=np.zeros(n2 * ns))
    L, pp = ob.lib(), C.byref(p)
    for it in range(1, 3):
        p.istep0 = p.istep = 1
        p.itn = it
        rt.set_params(p)
        for who, a in arrs.items():
            for nsp in range(ns):
                sl = slice(nsp * n2, (nsp + 1) * n2)
                qv = a["q"].reshape(p.nq, ns * n2)[:, sl].ravel()   # time_step of one instance
                ts, bt = np.zeros(n2), np.zeros(n2)
                p1 = type(p).from_buffer_copy(p)
                p1.nspec = 1
                L.oro_time_step(C.byref(p1), ob.ptr(np.ascontiguousarray(qv)), ob.ptr(c.xx), ob.ptr(c.xy),
                                ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(ts), ob.ptr(bt),
                                ob.ptr(c.iblank))
                a["tscale"][sl], a["bt"][sl] = ts, bt
            if who == "oracle":
                norms, loc = np.zeros(3 * ns), np.zeros(3 * ns, dtype=np.int32)
                st = L.oro_step_u(pp, ob.ptr(a["q"]), ob.ptr(a["s"]), ob.ptr(x), ob.ptr(y), ob.ptr(xv), ob.ptr(yv),
                                  ob.ptr(iblank), ob.ptr(xx), ob.ptr(xy), ob.ptr(yx), ob.ptr(yy), ob.ptr(ug),
                                  ob.ptr(vg), ob.ptr(ugv), ob.ptr(vgv), ob.ptr(a["turmu"]), ob.ptr(a["tscale"]),
                                  ob.ptr(a["bt"]), ob.ptr(Ds), ob.ptr(norms), ob.ptr(loc), ob.ptr(qnewt), None, None,
                                  None, None)
                assert st == 0
            else:
                rt.step(a["q"], None, None, qnewt, a["s"], x, y, xv, yv, iblank, xx, xy, yx, yy, ug, vg, ugv, vgv,
                        None, None, None, None, a["turmu"], a["tscale"], a["bt"], Ds, 1, p.jd, p.kd)
        assert relerr(arrs["gpu"]["q"], arrs["oracle"]["q"]) <= 1e-12
    # the Newton term changed the trajectory
    p0 = type(p).from_buffer_copy(p)
    assert not np.array_equal(arrs["gpu"]["q"], q)
