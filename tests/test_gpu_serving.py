"""Serving: admission by device memory, with requests queued until
retirements free enough of the solver's budget.

A request's footprint is ot2d_instance_bytes (all its device arrays); the
solver admits a request when it fits the budget next to the live ones,
queues it in submission order otherwise, and refuses one larger than the
whole budget.  Queued requests start later but compute exactly what they
compute alone."""
import numpy as np
import pytest

from turns2d_urans_git_gb300 import api
from turns2d_urans_git_gb300.abi import OT2D_ERR_NOMEM, OT2D_FP32_MIXED, OT2D_FP64, OT2D_OPT_BUDGET_MB

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
def test_footprint_admission_queues_and_matches_solo(precision, tmp_path):
    case = api.config_c2(jmax=129, kmax=33, fsmach=0.4, alfa=2.0, rey=2e6, ds_wall=1e-4)
    _, prm, xv, yv = case
    nbytes = api.instance_bytes(prm, precision)
    mib = (5 * nbytes // 2 + (1 << 20) - 1) >> 20          # room for two requests, not three
    assert 2 * nbytes <= mib << 20 < 3 * nbytes
    nsteps = 30
    solo = api.Solver(precision, check_every=10, keep_q=True)
    sid = solo.add(prm, xv, yv, orders=0.0, max_iters=nsteps)
    solo.iterate(nsteps)
    solo.sync()
    q_solo, r_solo = solo.get_q(sid, prm), solo.result(sid)
    solo.close()

    sv = api.Solver(precision, check_every=10, keep_q=True)
    sv.set_option(OT2D_OPT_BUDGET_MB, mib)
    log = str(tmp_path / "requests.jsonl")
    sv.set_log(log)
    ids = [sv.add(prm, xv, yv, orders=0.0, max_iters=nsteps) for _ in range(5)]
    assert sv.queued() == 3
    assert sv.live() == 5
    assert sv.device_bytes() == 2 * nbytes
    rs = [sv.result(i) for i in ids]
    assert all(r.t_admit >= 0 for r in rs[:2]) and all(r.t_admit < 0 for r in rs[2:])
    # a request larger than the whole budget is refused
    big = api.config_c2(jmax=513, kmax=129)
    with pytest.raises(RuntimeError, match=r"failed \(%d\)" % OT2D_ERR_NOMEM):
        sv.add(big[1], big[2], big[3], orders=0.0, max_iters=nsteps)
    while sv.live() > 0:
        sv.iterate(nsteps)
        assert sv.device_bytes() <= mib << 20
    sv.sync()
    rs = [sv.result(i) for i in ids]
    # admitted in submission order, two at a time, as memory was freed
    adm = [r.t_admit for r in rs]
    assert all(a >= 0 for a in adm) and adm == sorted(adm)
    assert rs[2].t_admit >= rs[0].t_done and rs[4].t_admit >= rs[2].t_done
    for i, r in zip(ids, rs):
        assert r.status == 0 and r.iterations == nsteps
        assert r.t_submit <= r.t_admit <= r.t_done
        assert np.array_equal(sv.get_q(i, prm), q_solo)
        assert r.cl == r_solo.cl and r.cd == r_solo.cd
    sv.close()
    # the per-request log: one JSON line per retired request
    import json
    recs = [json.loads(line) for line in open(log)]
    assert sorted(x["id"] for x in recs) == sorted(ids)
    for x in recs:
        r = rs[ids.index(x["id"])]
        assert x["status"] == 0 and x["iterations"] == nsteps and x["cl"] == r.cl
        assert x["t_submit"] <= x["t_admit"] <= x["t_done"] and (x["jmax"], x["kmax"]) == (prm.jmax, prm.kmax)
