"""Failure handling of the batched solver, with the faults made on the host.

The reference stops the whole run on a bad state (monitor, step.f:332-392 ->
Turns_overset.f:495-497) or a blown-up norm (step.f:104-110).  The batched
solver retires only the request that failed and keeps the others going:

* a request admitted with a NaN or a negative-pressure cell in its state
  retires with OT2D_ERR_MONITOR or OT2D_ERR_NORM, and every other request of
  the batch keeps the bits of its solo run;
* with the LU-SGS sweep's wait limit lowered to one poll, the waits run out:
  the kernel returns, the instance retires with OT2D_ERR_TIMEOUT, and the
  device stays usable for the next request.

No GPU fault, trap or hang is involved: the bad values are ordinary data, and
every device wait is bounded."""
import numpy as np
import pytest

from turns2d_urans_git_gb300 import api
from turns2d_urans_git_gb300.abi import (OT2D_ERR_MONITOR, OT2D_ERR_NORM, OT2D_ERR_TIMEOUT, OT2D_FP32_MIXED,
                                         OT2D_FP64, OT2D_OPT_POLL_LIMIT)

pytestmark = pytest.mark.gpu

NSTEPS = 40


def _cases():
    return [api.config_c2(jmax=97, kmax=33, fsmach=0.4, alfa=2.0, rey=2e6, ds_wall=1e-4),
            api.config_c1(jmax=97, kmax=25),
            api.config_c2(jmax=65, kmax=25, fsmach=0.5, alfa=1.0, rey=2e6, ds_wall=1e-4),
            api.config_c2(jmax=129, kmax=33, fsmach=0.3, alfa=4.0, rey=3e6, ds_wall=1e-4)]


def _solo(precision, case):
    _, prm, xv, yv = case
    sv = api.Solver(precision, check_every=10, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=NSTEPS)
    sv.iterate(NSTEPS)
    sv.sync()
    r, q = sv.result(iid), sv.get_q(iid, prm)
    sv.close()
    return r, q


def _freestream_state(precision, case):
    _, prm, xv, yv = case
    sv = api.Solver(precision, check_every=10, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=NSTEPS)
    q = sv.get_q(iid, prm)
    sv.close()
    return q


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
@pytest.mark.parametrize("fault", ["nan", "negative_pressure"])
def test_bad_request_retires_alone(fault, precision):
    cases = _cases()
    bad = 2
    solo = {i: _solo(precision, c) for i, c in enumerate(cases) if i != bad}
    _, prm, xv, yv = cases[bad]
    q = _freestream_state(precision, cases[bad])
    jd, kd, qs = prm.jd, prm.kd, prm.jd * prm.kd * prm.nspec
    o = (kd // 2 - 1) * jd + (jd // 2 - 1)          # an interior cell
    if fault == "nan":
        q[1 * qs + o] = np.nan                       # rho*u / J
    else:
        q[3 * qs + o] = -abs(q[3 * qs + o])          # energy / J < 0: p < 0
    sv = api.Solver(precision, check_every=10, keep_q=True)
    ids = {}
    for i, (_, p_, x_, y_) in enumerate(cases):
        ids[i] = (sv.add_state(p_, x_, y_, q, orders=0.0, max_iters=NSTEPS) if i == bad
                  else sv.add(p_, x_, y_, orders=0.0, max_iters=NSTEPS))
    sv.iterate(NSTEPS)
    sv.sync()
    rb = sv.result(ids[bad])
    assert rb.status in (OT2D_ERR_MONITOR, OT2D_ERR_NORM), rb.status
    assert rb.iterations < NSTEPS and not rb.converged
    for i, (r0, q0) in solo.items():
        r = sv.result(ids[i])
        assert r.status == 0 and r.iterations == NSTEPS
        assert np.array_equal(sv.get_q(ids[i], cases[i][1]), q0)
        assert r.cl == r0.cl and r.cd == r0.cd and r.rsum_last == r0.rsum_last
    sv.close()


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
def test_sweep_wait_runs_out_and_retires_with_timeout(precision):
    """97 x 69 vertices: 68 interior rows, three 32-row bands per sweep, so
    every band but the first waits for its neighbour's progress; one poll is
    never enough.  Afterwards the default limit is restored and a new
    request on the same solver runs to its solo result."""
    _, prm, xv, yv = api.config_c1(jmax=97, kmax=69)
    sv = api.Solver(precision, check_every=1, keep_q=True)
    sv.set_option(OT2D_OPT_POLL_LIMIT, 1)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=5)
    sv.iterate(3)
    sv.sync()
    r = sv.result(iid)
    assert r.status == OT2D_ERR_TIMEOUT, r.status
    assert r.iterations <= 3 and not r.converged
    assert sv.live() == 0
    # the kernel returned and left the state alone: the interior is finite
    assert np.all(np.isfinite(sv.get_q(iid, prm)))
    sv.set_option(OT2D_OPT_POLL_LIMIT, 1 << 22)
    case = api.config_c1(jmax=97, kmax=69)
    r0, q0 = _solo(precision, case)
    sv.set_option(1, 10)
    iid2 = sv.add(case[1], case[2], case[3], orders=0.0, max_iters=NSTEPS)
    sv.iterate(NSTEPS)
    sv.sync()
    r2 = sv.result(iid2)
    assert r2.status == 0 and r2.iterations == NSTEPS
    assert np.array_equal(sv.get_q(iid2, case[1]), q0)
    sv.close()


def test_solvers_on_two_devices():
    """One process driving two GPUs: every kernel attribute (dynamic shared
    memory limits above 48 KB) is set per device, so the second device's
    solves run too."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    case = api.config_c2(jmax=97, kmax=33, fsmach=0.4, alfa=2.0, rey=2e6, ds_wall=1e-4)
    _, prm, xv, yv = case
    out = []
    for dev in (0, 1):
        sv = api.Solver(OT2D_FP64, device=dev, check_every=10, keep_q=True)
        iid = sv.add(prm, xv, yv, orders=0.0, max_iters=20)
        sv.iterate(20)
        sv.sync()
        r = sv.result(iid)
        assert r.status == 0 and r.iterations == 20
        out.append(sv.get_q(iid, prm))
        sv.close()
    assert np.array_equal(out[0], out[1])
