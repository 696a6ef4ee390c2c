"""ot2d_norms_noalloc: the residual norms of step.f:58-93 computed with
static device scratch, against the norms ot2d_step reports for the same
residual.  Collected last (file name) so that it also runs after every other
test in the same process; it passes alone as well."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import Case, relerr
from turns2d_urans_git_gb300 import routines as rt
from turns2d_urans_git_gb300.api import lib

pytestmark = pytest.mark.gpu


def _residual_and_step_norms(c):
    """The residual ot2d_step takes its norms of (bc, then s = 0 and rhsup,
    + visrhs when viscous), and the norms ot2d_step itself reports."""
    rt.set_params(c.p)
    q, ts, bt = c.q.copy(), np.zeros(c.n2), np.zeros(c.n2)
    rt.time_step(q, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, ts, bt, c.iblank, c.jd, c.kd)
    q_step, s_step, turmu = q.copy(), np.zeros(c.n2 * c.p.nv), c.turmu.copy()
    nm = rt.step(q_step, None, None, None, s_step, c.x, c.y, c.xv, c.yv, c.iblank, c.xx, c.xy, c.yx, c.yy, c.ug,
                 c.vg, c.ugv, c.vgv, None, None, None, None, turmu, ts, bt, np.zeros(1), 1, c.jd, c.kd)
    rt.bc(q, c.x, c.y, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, 1, c.jd, c.kd, bt)
    s = np.zeros(c.n2 * c.p.nv)
    rt.rhsup(q, s, c.xx, c.xy, c.yx, c.yy, c.x, c.y, c.xv, c.yv, c.xv, c.yv, c.xv, c.yv, c.iblank, c.ugv, c.vgv,
             c.jd, c.kd, 1, 1, bt)
    if not c.p.invisc:
        rt.visrhs(c.turmu.copy(), q, s, c.xx, c.xy, c.yx, c.yy, c.ug, c.vg, ts, c.iblank, c.jd, c.kd)
    return s, np.asarray(nm[:3])


@pytest.mark.parametrize("visc", [False, True])
def test_norms_noalloc_matches_step(visc):
    torch = pytest.importorskip("torch")
    c = Case(viscous=visc, seed=21, perturb=0.01)
    s, ref = _residual_and_step_norms(c)
    d_s = torch.from_numpy(s).cuda()
    d_ib = torch.from_numpy(c.iblank).cuda()
    torch.cuda.synchronize()
    f = lib().ot2d_norms_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p] + [C.c_int32] * 7 + [C.c_void_p, C.c_void_p]
    p = c.p
    outs = []
    for _ in range(2):  # two calls in a row reuse the same scratch
        out = np.zeros(6)
        rc = f(d_s.data_ptr(), d_ib.data_ptr(), p.jd, p.kd, p.jbeg, p.jend, p.kbeg, p.kend, p.nmv,
               out.ctypes.data, None)
        assert rc == 0
        outs.append(out)
    for out in outs:
        assert relerr(out[:3], ref) <= 1e-12
    assert np.array_equal(outs[0], outs[1])
    # the reported location holds the maximum
    j, k, n = (int(v) for v in outs[0][3:])
    sv = s.reshape(p.nv, p.kd, p.jd)
    assert abs(sv[n - 1, k - 1, j - 1]) == outs[0][2]


def test_norms_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    f = lib().ot2d_norms_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p] + [C.c_int32] * 7 + [C.c_void_p, C.c_void_p]
    out = np.zeros(6)
    d_s = torch.zeros(16, dtype=torch.float64, device="cuda")
    d_ib = torch.ones(16, dtype=torch.int32, device="cuda")
    # 2049 x 1025 array cells is above the 1,048,576-cell limit: rejected
    # (OT2D_ERR_ARG) before anything is launched
    rc = f(d_s.data_ptr(), d_ib.data_ptr(), 2049, 1025, 2, 2048, 2, 1024, 4, out.ctypes.data, None)
    assert rc == 1
    assert not out.any()


def _norms_numpy(s, iblank, jd, kd, js, je, ks, ke, nmv):
    """step.f:67-93 restated with numpy: rsum and resrho over jd*kd, resmax
    and the first location (loop order k, then n, then j) that holds it."""
    sv = s.reshape(-1, kd, jd)
    m = np.maximum(iblank.reshape(kd, jd), 0).astype(np.float64)[ks - 1:ke, js - 1:je]
    inner = sv[:, ks - 1:ke, js - 1:je]
    rsum = np.sqrt(sum(np.sum((inner[n] * m) ** 2) for n in range(4)) / float(jd * kd))
    resrho = np.sqrt(np.sum(inner[0] ** 2) / float(jd * kd))
    a = np.abs(inner[:nmv]) * m                      # (n, k, j)
    resmax = a.max()
    order = np.transpose(a, (1, 0, 2)).ravel()       # k, then n, then j
    i = int(np.argmax(order == resmax))              # first occurrence
    k, rest = divmod(i, nmv * (je - js + 1))
    n, j = divmod(rest, je - js + 1)
    return rsum, resrho, resmax, (j + js, k + ks, n + 1)


def test_norms_noalloc_at_capacity_on_a_stream():
    """The largest accepted array (1025 x 1023 = 1,048,575 cells, 4096 blocks:
    the static scratch's capacity, so the final pass walks 128 partials per
    lane), a residual with a planted tie for the maximum and masked cells,
    run on an explicit stream twice in a row."""
    torch = pytest.importorskip("torch")
    jd, kd, nmv, nv = 1025, 1023, 4, 5
    js, je, ks, ke = 2, jd - 1, 2, kd - 1
    rng = np.random.default_rng(5)
    s = rng.standard_normal(nv * kd * jd)
    ib = np.where(rng.random(kd * jd) < 0.05, rng.integers(-1, 1, kd * jd), 1).astype(np.int32)
    sv, ibv = s.reshape(nv, kd, jd), ib.reshape(kd, jd)
    big = 50.0
    # masked cells earlier in loop order than the maximum do not count
    ibv[3, 10] = 0; sv[0, 3, 10] = 2 * big
    ibv[4, 11] = -1; sv[1, 4, 11] = -2 * big
    # the same maximum at three places: the first in (k, n, j) order wins
    for (n, k, j) in ((2, 700, 40), (1, 700, 900), (0, 900, 3)):
        ibv[k - 1, j - 1] = 1
        sv[n, k - 1, j - 1] = big if n != 1 else -big
    assert int(np.count_nonzero(np.abs(sv[:nmv, ks - 1:ke, js - 1:je]) * np.maximum(ibv, 0)[ks - 1:ke, js - 1:je]
                                == big)) == 3
    ref = _norms_numpy(s, ib, jd, kd, js, je, ks, ke, nmv)
    assert ref[3] == (900, 700, 2)
    f = lib().ot2d_norms_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p] + [C.c_int32] * 7 + [C.c_void_p, C.c_void_p]
    d_s = torch.from_numpy(s).cuda()
    d_ib = torch.from_numpy(ib).cuda()
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    outs = []
    for _ in range(2):
        out = np.zeros(6)
        rc = f(d_s.data_ptr(), d_ib.data_ptr(), jd, kd, js, je, ks, ke, nmv, out.ctypes.data, st.cuda_stream)
        assert rc == 0
        outs.append(out)
    for out in outs:
        assert relerr(out[:2], np.array(ref[:2])) <= 1e-12
        assert out[2] == ref[2]
        assert tuple(int(v) for v in out[3:]) == ref[3]
    assert np.array_equal(outs[0], outs[1])
