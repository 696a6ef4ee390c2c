"""GPU parity of every drop-in routine and of the batched solver against the
CPU FP64 oracle, through the C-ABI (numpy host arrays staged by the
library, registered host arrays, and CUDA device pointers).

Tolerance: the plain FP64 path must agree with the oracle to 1e-12 relative
(the bound the path is specified to); most routines are bit-exact because the FP64 kernels
keep the reference's operation order without fused multiply-adds and IEEE
division / square root are correctly rounded on both sides.  pow/exp in the
SA source term may differ by an ulp.
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


def _o(c):
    return C.byref(c.p)


def test_time_step():
    for visc in (False, True):
        c = Case(viscous=visc, seed=1)
        ts_o, bt_o = np.zeros(c.n2), np.zeros(c.n2)
        ob.lib().oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                               ob.ptr(c.vg), ob.ptr(ts_o), ob.ptr(bt_o), ob.ptr(c.iblank))
        rt.set_params(c.p)
        ts, bt = np.zeros(c.n2), np.zeros(c.n2)
        rt.time_step(c.q, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, ts, bt, c.iblank, c.jd, c.kd)
        assert relerr(ts, ts_o) <= TOL and relerr(bt, bt_o) <= TOL


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("istep0", [1, 12, 40])
def test_bc(visc, istep0):
    c = Case(viscous=visc, seed=2, istep0=istep0)
    qo = c.q.copy()
    ob.lib().oro_bc(_o(c), ob.ptr(qo), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                    ob.ptr(c.vg), ob.ptr(c.bt))
    rt.set_params(c.p)
    q = c.q.copy()
    rt.bc(q, c.x, c.y, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, 1, c.jd, c.kd, c.bt)
    assert relerr(q, qo) <= TOL
    assert not np.array_equal(qo, c.q)  # the halo really changed


@pytest.mark.parametrize("ilim,irhsy", [(0, -3), (1, -3), (1, -2), (4, -3), (1, -1), (2, -3), (-2, -2), (2, -1)])
def test_rhsup(ilim, irhsy):
    c = Case(ilim=ilim, irhsy=irhsy, seed=3)
    so = np.random.default_rng(9).uniform(-1, 1, c.n2 * c.p.nv) * 1e-3
    s = so.copy()
    ob.lib().oro_rhsup(_o(c), ob.ptr(c.q), ob.ptr(so), ob.ptr(c.xv), ob.ptr(c.yv), ob.ptr(c.iblank), ob.ptr(c.ugv),
                       ob.ptr(c.vgv))
    rt.set_params(c.p)
    rt.rhsup(c.q, s, c.xx, c.xy, c.yx, c.yy, c.x, c.y, c.xv, c.yv, c.xv, c.yv, c.xv, c.yv, c.iblank, c.ugv, c.vgv,
             c.jd, c.kd, 1, 1, c.bt)
    assert relerr(s, so) <= TOL


def test_visrhs():
    c = Case(viscous=True, seed=4)
    so = np.zeros(c.n2 * c.p.nv)
    s = so.copy()
    ob.lib().oro_visrhs(_o(c), ob.ptr(c.turmu), ob.ptr(c.q), ob.ptr(so), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx),
                        ob.ptr(c.yy))
    rt.set_params(c.p)
    rt.visrhs(c.turmu, c.q, s, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.tscale, c.iblank, c.jd, c.kd)
    assert np.abs(so).max() > 0
    assert relerr(s, so) <= TOL


def test_rbc():
    c = Case(seed=5)
    so = np.random.default_rng(2).uniform(-1, 1, c.n2 * c.p.nv)
    s = so.copy()
    ob.lib().oro_rbc(_o(c), ob.ptr(c.q), ob.ptr(so))
    rt.set_params(c.p)
    rt.rbc(c.q, s, c.x, c.y, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, 1, c.jd, c.kd, c.bt)
    assert np.array_equal(s, so)


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("size", [(65, 25), (97, 69)])
def test_ilu2d(visc, size):
    """ilu2d (lhs.f:470-814) drop-in against the oracle.  65x25: one band of
    24 rows (every step in the sweep's per-step form); 97x69: two full bands
    of 32 rows, whose steps 32..95 run as steady groups, and a band of 4
    rows, so the cross-band hand-offs go steady -> steady -> per-step
    (forward) and back (backward)."""
    c = Case(jmax=size[0], kmax=size[1], viscous=visc, seed=6)
    L = ob.lib()
    L.oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                    ob.ptr(c.vg), ob.ptr(c.tscale), ob.ptr(c.bt), ob.ptr(c.iblank))
    so = np.random.default_rng(3).uniform(-1, 1, c.n2 * c.p.nv) * 1e-4
    s, qo, q = so.copy(), c.q.copy(), c.q.copy()
    L.oro_ilu2d(_o(c), ob.ptr(qo), ob.ptr(so), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                ob.ptr(c.vg), ob.ptr(c.turmu), ob.ptr(c.tscale))
    rt.set_params(c.p)
    p = c.p
    rt.ilu2d(q, s, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.turmu, c.tscale)
    assert relerr(s, so) <= TOL
    assert relerr(q, qo) <= TOL


def test_vmu_sa():
    c = Case(viscous=True, seed=7)
    L = ob.lib()
    L.oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                    ob.ptr(c.vg), ob.ptr(c.tscale), ob.ptr(c.bt), ob.ptr(c.iblank))
    s = np.zeros(c.n2 * c.p.nv)
    qo, q, to, t = c.q.copy(), c.q.copy(), c.turmu.copy(), c.turmu.copy()
    L.oro_vmu_sa(_o(c), ob.ptr(qo), ob.ptr(s), ob.ptr(to), ob.ptr(c.x), ob.ptr(c.y), ob.ptr(c.xv), ob.ptr(c.yv),
                 ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(c.tscale),
                 ob.ptr(c.iblank))
    rt.set_params(c.p)
    rt.vmu_sa(q, s, t, c.x, c.y, c.xv, c.yv, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.jd, c.kd, c.tscale, c.iblank, 1, 1)
    n5 = slice(4 * c.n2, 5 * c.n2)
    assert not np.array_equal(qo[n5], c.q[n5])
    assert relerr(q[n5], qo[n5]) <= TOL
    assert relerr(t, to) <= TOL


def test_komegasst():
    """komegasst (k-omega SST, komegasst.f:2-187) on a perturbed state,
    drop-in against the oracle; the BC ramp is mid-way (istep0 = 10)."""
    c = Case(viscous=True, seed=17, iturb=2)
    L = ob.lib()
    L.oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                    ob.ptr(c.vg), ob.ptr(c.tscale), ob.ptr(c.bt), ob.ptr(c.iblank))
    so = np.random.default_rng(5).uniform(-1, 1, c.n2 * c.p.nv) * 1e-6
    s = so.copy()
    qo, q, to, t = c.q.copy(), c.q.copy(), c.turmu.copy(), c.turmu.copy()
    L.oro_komegasst(_o(c), ob.ptr(qo), ob.ptr(so), ob.ptr(to), ob.ptr(c.x), ob.ptr(c.y), ob.ptr(c.xv), ob.ptr(c.yv),
                    ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug), ob.ptr(c.vg),
                    ob.ptr(c.tscale), ob.ptr(c.iblank), None)
    rt.set_params(c.p)
    rt.komegasst(q, s, t, c.x, c.y, c.xv, c.yv, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.jd, c.kd, c.tscale, c.iblank, 1)
    kw = slice(4 * c.n2, 6 * c.n2)
    assert not np.array_equal(qo[kw], c.q[kw])
    assert relerr(q[kw], qo[kw]) <= TOL
    assert relerr(t, to) <= TOL
    assert relerr(s[kw], so[kw]) <= TOL


def test_solver_sst_fp64_matches_oracle():
    """The batched solver on a k-omega SST case (cambered NACA 2412, WENO +
    Roe, LU-SGS), 40 iterations, FP64, against the oracle driver."""
    _, prm, xv, yv = api.cmesh_case(97, 33, naca=(0.02, 0.4, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=2,
                                    irhsy=-3, ilim=4, ilhs=1, iconstant_cfl=1, dt=20.0, fsmach=0.73, alfa=2.8,
                                    rey=6.5e6)
    r, q, hist, forces, q_o = _solver_vs_oracle(prm, xv, yv, 40, OT2D_FP64)
    assert r.status == 0 and r.iterations == 40
    assert abs(r.rsum_last - hist[-1, 0]) <= 1e-10 * hist[-1, 0]
    assert relerr(q, q_o) <= 1e-10
    f = forces[0]
    for a, b in ((r.cl, f[0]), (r.cd, f[1]), (r.cm, f[2])):
        assert abs(a - b) <= 1e-10 * max(abs(b), 1e-3)


@pytest.mark.parametrize("visc,ilhs", [(False, 2), (True, 2), (True, 3)])
def test_arc2d(visc, ilhs):
    """arc2d (diagonalised ADI, lhs.f:817-1057) with the pentadiagonal
    (ilhs 2) or upwind tridiagonal (ilhs 3) line inversions, on a perturbed
    state and a random right-hand side."""
    c = Case(viscous=visc, seed=19)
    c.p.ilhs = ilhs
    L = ob.lib()
    L.oro_time_step(_o(c), ob.ptr(c.q), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                    ob.ptr(c.vg), ob.ptr(c.tscale), ob.ptr(c.bt), ob.ptr(c.iblank))
    so = np.random.default_rng(23).uniform(-1, 1, c.n2 * c.p.nv) * 1e-4
    s = so.copy()
    qo, q = c.q.copy(), c.q.copy()
    L.oro_arc2d(_o(c), ob.ptr(qo), ob.ptr(so), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy), ob.ptr(c.ug),
                ob.ptr(c.vg), ob.ptr(c.turmu), ob.ptr(c.iblank), ob.ptr(c.tscale), ob.ptr(c.bt))
    rt.set_params(c.p)
    p = c.p
    rt.arc2d(q, s, c.jd, c.kd, p.jbeg, p.jend, p.kbeg, p.kend, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, c.turmu, c.iblank,
             c.tscale, c.bt)
    assert relerr(s[:4 * c.n2], so[:4 * c.n2]) <= TOL
    assert relerr(q, qo) <= TOL


@pytest.mark.parametrize("kind", ["euler", "euler_up", "sst_weno"])
def test_solver_adi_fp64_matches_oracle(kind):
    """The batched solver with the ADI operator (ilhs = 2, or 3 for the
    upwind variant), FP64, against the oracle driver: inviscid cases and a
    k-omega SST + WENO case."""
    if kind.startswith("euler"):
        _, prm, xv, yv = api.cmesh_case(97, 25, ds_wall=2e-3, invisc=1, lamin=1, irhsy=-3, ilim=1,
                                        ilhs=3 if kind == "euler_up" else 2, iconstant_cfl=1, dt=2.0, fsmach=0.8,
                                        alfa=1.25)
    else:
        _, prm, xv, yv = api.cmesh_case(97, 33, naca=(0.02, 0.4, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=2,
                                        irhsy=-3, ilim=4, ilhs=2, iconstant_cfl=1, dt=2.0, fsmach=0.73, alfa=2.8,
                                        rey=6.5e6)
    r, q, hist, forces, q_o = _solver_vs_oracle(prm, xv, yv, 40, OT2D_FP64)
    assert r.status == 0 and r.iterations == 40
    assert abs(r.rsum_last - hist[-1, 0]) <= 1e-10 * hist[-1, 0]
    assert relerr(q, q_o) <= 1e-10


@pytest.mark.parametrize("nspec", [3, 5])
def test_timespectralrhs(nspec):
    """sources.f:2-27: s(nsp) -= rotf * sum_m Ds(m,nsp) q(m), every instance."""
    _, p, _, _ = api.cmesh_case(65, 25, invisc=1, lamin=1, timespectral=1, nspec=nspec, rf=0.1, angmax=5.0,
                                xac=0.25, motiontype=1, fsmach=0.3)
    rng = np.random.default_rng(nspec)
    n2 = p.jd * p.kd
    q = rng.uniform(0.5, 1.5, n2 * nspec * p.nq)
    s0 = rng.uniform(-1, 1, n2 * nspec * p.nv) * 1e-3
    Ds = np.zeros(nspec * nspec)
    ob.lib().oro_computeTScoefs(nspec, ob.ptr(Ds))
    rt.set_params(p)
    for nsp in range(1, nspec + 1):
        so, s = s0.copy(), s0.copy()
        ob.lib().oro_timespectralrhs(C.byref(p), ob.ptr(q), ob.ptr(so), ob.ptr(Ds), nsp)
        rt.timespectralrhs(q, s, Ds, p.jd, p.kd, nsp)
        assert not np.array_equal(so, s0)
        assert relerr(s, so) <= TOL


@pytest.mark.parametrize("visc", [False, True])
def test_solver_ts_fp64_matches_oracle(visc):
    """A time-spectral pitching-airfoil request (3 instances coupled through
    Ds, pitching grids and grid speeds) through the batched solver, FP64,
    against the oracle driver."""
    kw = dict(timespectral=1, nspec=3, rf=0.1, angmax=5.0, xac=0.25, motiontype=1, fsmach=0.3, alfa=2.0,
              irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1)
    if visc:
        _, prm, xv, yv = api.cmesh_case(97, 33, ds_wall=1e-3, invisc=0, lamin=0, iturb=1, dt=20.0, rey=2e6,
                                        vnuinf=3.0, **kw)
    else:
        _, prm, xv, yv = api.cmesh_case(97, 25, ds_wall=2e-3, invisc=1, lamin=1, dt=10.0, **kw)
    r, q, hist, forces, q_o = _solver_vs_oracle(prm, xv, yv, 30, OT2D_FP64)
    assert r.status == 0 and r.iterations == 30
    assert relerr(q, q_o) <= 1e-10


def _full_arrays(c):
    return dict(q=c.q.copy(), s=np.zeros(c.n2 * c.p.nv), turmu=c.turmu.copy(), tscale=np.zeros(c.n2),
                bt=np.zeros(c.n2))


@pytest.mark.parametrize("visc", [False, True])
def test_step(visc):
    """step.f: bc, residual, norms, rbc, LU-SGS, SA, update -- three
    consecutive calls, each preceded by time_step."""
    c = Case(viscous=visc, seed=8, perturb=0.01)
    a, b = _full_arrays(c), _full_arrays(c)
    L = ob.lib()
    rt.set_params(c.p)
    for it in range(3):
        c.p.istep0 = it + 1
        c.p.istep = it + 1
        rt.set_params(c.p)
        for arr, gpu in ((a, False), (b, True)):
            if gpu:
                rt.time_step(arr["q"], c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, arr["tscale"], arr["bt"], c.iblank, c.jd, c.kd)
                nm = rt.step(arr["q"], None, None, None, arr["s"], c.x, c.y, c.xv, c.yv, c.iblank, c.xx, c.xy, c.yx,
                             c.yy, c.ug, c.vg, c.ugv, c.vgv, None, None, None, None, arr["turmu"], arr["tscale"],
                             arr["bt"], np.zeros(1), 1, c.jd, c.kd)
                norms_g = nm[:3]
            else:
                L.oro_time_step(_o(c), ob.ptr(arr["q"]), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy),
                                ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(arr["tscale"]), ob.ptr(arr["bt"]), ob.ptr(c.iblank))
                norms_o = np.zeros(3)
                loc = np.zeros(3, dtype=np.int32)
                st = L.oro_step(_o(c), ob.ptr(arr["q"]), ob.ptr(arr["s"]), ob.ptr(c.x), ob.ptr(c.y), ob.ptr(c.xv),
                                ob.ptr(c.yv), ob.ptr(c.iblank), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx), ob.ptr(c.yy),
                                ob.ptr(c.ug), ob.ptr(c.vg), ob.ptr(c.ugv), ob.ptr(c.vgv), ob.ptr(arr["turmu"]),
                                ob.ptr(arr["tscale"]), ob.ptr(arr["bt"]), ob.ptr(np.zeros(1)), ob.ptr(norms_o),
                                ob.ptr(loc))
                assert st == 0
        assert relerr(norms_g, norms_o) <= 1e-12
        assert relerr(b["q"], a["q"]) <= TOL
        assert relerr(b["turmu"], a["turmu"]) <= TOL


def test_monitor_flags_bad_state():
    c = Case(seed=9)
    rt.set_params(c.p)
    assert rt.monitor(c.q, c.jd, c.kd) == 0
    q = c.q.copy()
    q.reshape(c.p.nq, -1)[3, 40] = -1.0  # negative energy -> negative a^2
    assert rt.monitor(q, c.jd, c.kd) == 1
    assert ob.lib().oro_monitor(_o(c), ob.ptr(q)) > 0


@pytest.mark.parametrize("visc", [False, True])
def test_force2d(visc):
    c = Case(viscous=visc, seed=10)
    out = np.zeros(4)
    ob.lib().oro_force2d(_o(c), ob.ptr(c.q), ob.ptr(c.xv), ob.ptr(c.yv), ob.ptr(c.xx), ob.ptr(c.xy), ob.ptr(c.yx),
                         ob.ptr(c.yy), ob.ptr(out))
    rt.set_params(c.p)
    g = rt.force2d(c.jd, c.kd, c.x, c.y, c.xv, c.yv, c.q, c.xx, c.xy, c.yx, c.yy)
    assert relerr(np.array(g), out) <= TOL


def _solver_vs_oracle(prm, xv, yv, nsteps, precision):
    n, hist, forces, q_o = ob.solve(prm, xv.ravel(), yv.ravel(), nsteps)
    assert n == nsteps
    sv = api.Solver(precision, check_every=nsteps, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=nsteps)
    sv.iterate(nsteps)
    sv.sync()
    r = sv.result(iid)
    q = sv.get_q(iid, prm)
    sv.close()
    return r, q, hist, forces, q_o


@pytest.mark.parametrize("kind", ["c1", "c2"])
def test_solver_fp64_matches_oracle(kind):
    if kind == "c1":
        _, prm, xv, yv = api.config_c1(jmax=97, kmax=25)
    else:
        _, prm, xv, yv = api.config_c2(jmax=97, kmax=33, ds_wall=1e-4)
    r, q, hist, forces, q_o = _solver_vs_oracle(prm, xv, yv, 60, OT2D_FP64)
    assert r.status == 0 and r.iterations == 60
    assert abs(r.rsum_last - hist[-1, 0]) <= 1e-10 * hist[-1, 0]
    assert abs(r.rsum_first - hist[0, 0]) <= 1e-12 * hist[0, 0]
    assert relerr(q, q_o) <= 1e-10
    f = forces[0]
    for a, b in ((r.cl, f[0]), (r.cd, f[1]), (r.cm, f[2])):
        assert abs(a - b) <= 1e-10 * max(abs(b), 1e-3)


@pytest.mark.parametrize("kind", ["euler", "sa"])
def test_solver_quad_fp64_matches_oracle(kind):
    """The piecewise quadratic reconstruction (ilim 2: quad and tridag,
    eulerrhs.f:1233-1588) through the batched solver: k_quad's line solves
    and the residual's faces against the oracle.  The FP32-mixed path on
    the same request stays close to it."""
    if kind == "euler":
        _, prm, xv, yv = api.cmesh_case(97, 25, ds_wall=2e-3, invisc=1, lamin=1, irhsy=-3, ilim=2, ilhs=1,
                                        iconstant_cfl=1, dt=10.0, fsmach=0.5, alfa=1.25)
        tol = 1e-10
    else:
        _, prm, xv, yv = api.cmesh_case(97, 33, ds_wall=1e-4, invisc=0, lamin=0, iturb=1, irhsy=-3, ilim=2, ilhs=1,
                                        iconstant_cfl=1, dt=20.0, fsmach=0.3, alfa=2.0, rey=2e6, vnuinf=3.0)
        tol = 1e-9
    r, q, hist, forces, q_o = _solver_vs_oracle(prm, xv, yv, 40, OT2D_FP64)
    assert r.status == 0 and r.iterations == 40
    assert abs(r.rsum_last - hist[-1, 0]) <= tol * hist[-1, 0]
    assert relerr(q, q_o) <= tol
    f = forces[0]
    for a, b in ((r.cl, f[0]), (r.cd, f[1]), (r.cm, f[2])):
        assert abs(a - b) <= tol * max(abs(b), 1e-3)
    r32, q32, _, _, _ = _solver_vs_oracle(prm, xv, yv, 40, OT2D_FP32_MIXED)
    assert r32.status == 0 and relerr(q32, q_o) < 1e-3


def test_solver_fp32_mixed_close_to_fp64():
    _, prm, xv, yv = api.config_c1(jmax=97, kmax=25)
    r, q, hist, forces, q_o = _solver_vs_oracle(prm, xv, yv, 200, OT2D_FP32_MIXED)
    assert r.status == 0
    f = forces[0]
    assert abs(r.cl - f[0]) < 2e-3
    assert abs(r.cd - f[1]) < 5e-4
    assert relerr(q, q_o) < 1e-2


def test_batched_ragged_equals_solo():
    """A ragged batch (different sizes and flow conditions in one launch per
    kernel) gives every request exactly its solo FP64 result."""
    rng = np.random.default_rng(11)
    cases = [api.config_c2(jmax=j, kmax=k, fsmach=rng.uniform(0.3, 0.6), alfa=rng.uniform(-2, 6), rey=2e6,
                           ds_wall=1e-4) for (j, k) in ((65, 25), (97, 33), (129, 33))]
    cases.append(api.config_c1(jmax=97, kmax=25))
    nsteps = 40
    solo = []
    for (_, prm, xv, yv) in cases:
        sv = api.Solver(OT2D_FP64, check_every=nsteps, keep_q=True)
        iid = sv.add(prm, xv, yv, orders=0.0, max_iters=nsteps)
        sv.iterate(nsteps)
        sv.sync()
        solo.append((sv.result(iid), sv.get_q(iid, prm)))
        sv.close()
    sv = api.Solver(OT2D_FP64, check_every=nsteps, keep_q=True)
    ids = [sv.add(prm, xv, yv, orders=0.0, max_iters=nsteps) for (_, prm, xv, yv) in cases]
    sv.iterate(nsteps)
    sv.sync()
    for iid, (_, prm, _, _), (r0, q0) in zip(ids, cases, solo):
        r = sv.result(iid)
        assert np.array_equal(sv.get_q(iid, prm), q0)
        assert r.cl == r0.cl and r.cd == r0.cd and r.rsum_last == r0.rsum_last
    sv.close()


def test_device_pointers_and_registry():
    """The drop-in routines accept CUDA device pointers (used in place) and
    registered host arrays (device mirror, no copy) with identical results."""
    torch = pytest.importorskip("torch")
    c = Case(seed=12)
    rt.set_params(c.p)
    ts_h, bt_h = np.zeros(c.n2), np.zeros(c.n2)
    rt.time_step(c.q, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, ts_h, bt_h, c.iblank, c.jd, c.kd)
    dev = {k: torch.from_numpy(getattr(c, k)).cuda() for k in ("q", "xx", "xy", "yx", "yy", "ug", "vg", "iblank")}
    ts_d = torch.zeros(c.n2, dtype=torch.float64, device="cuda")
    bt_d = torch.zeros(c.n2, dtype=torch.float64, device="cuda")
    rt.time_step(dev["q"], dev["xx"], dev["xy"], dev["yx"], dev["yy"], dev["ug"], dev["vg"], ts_d, bt_d,
                 dev["iblank"], c.jd, c.kd)
    torch.cuda.synchronize()
    assert np.array_equal(ts_d.cpu().numpy(), ts_h)
    # registered host buffers: results land in the mirror until synced back
    L = api.lib()
    L.ot2d_register.argtypes = [C.c_void_p, C.c_size_t]
    L.ot2d_sync_to_host.argtypes = [C.c_void_p]
    L.ot2d_unregister.argtypes = [C.c_void_p]
    ts_r = np.zeros(c.n2)
    assert L.ot2d_register(C.c_void_p(ts_r.ctypes.data), ts_r.nbytes) == 0
    rt.time_step(c.q, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, ts_r, np.zeros(c.n2), c.iblank, c.jd, c.kd)
    assert not ts_r.any()
    assert L.ot2d_sync_to_host(C.c_void_p(ts_r.ctypes.data)) == 0
    assert np.array_equal(ts_r, ts_h)
    assert L.ot2d_unregister(C.c_void_p(ts_r.ctypes.data)) == 0
