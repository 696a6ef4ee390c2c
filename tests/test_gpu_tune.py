"""The autotuner's candidates on the GPU: every launch choice (residual tile
shape, LU-SGS copy group, LU-SGS band lag) gives the same state bit for bit,
in FP64 and in the FP32-mixed path (the L2 norm's partial sums follow the
tile shape, so the norms agree to rounding), and a tuning table handed to
the solver is applied to the batch of its size class."""
import json

import numpy as np
import pytest

from turns2d_urans_git_gb300 import api, tune
from turns2d_urans_git_gb300.abi import (OT2D_FP32_MIXED, OT2D_FP64, OT2D_OPT_LU_GROUP, OT2D_OPT_LU_LAG,
                                         OT2D_OPT_PIPELINE, OT2D_OPT_RT_SHAPE)

pytestmark = pytest.mark.gpu

NSTEPS = 12


def _run(precision, cases, choice=None, table=None):
    sv = api.Solver(precision, check_every=NSTEPS, keep_q=True)
    if choice is not None:
        shape, group, lag, pipe = choice
        sv.set_option(OT2D_OPT_RT_SHAPE, shape)
        sv.set_option(OT2D_OPT_LU_GROUP, group)
        sv.set_option(OT2D_OPT_LU_LAG, lag)
        sv.set_option(OT2D_OPT_PIPELINE, pipe)
    if table is not None:
        tune.apply(sv, table)
    ids = [sv.add(c[1], c[2], c[3], orders=0.0, max_iters=NSTEPS) for c in cases]
    sv.iterate(NSTEPS)
    sv.sync()
    out = [(sv.get_q(i, c[1]), sv.result(i)) for i, c in zip(ids, cases)]
    sv.close()
    return out


def _cases():
    # 97x69: three LU-SGS bands and ragged residual tiles in every shape;
    # an SA request and a WENO SST request share the batch
    return [api.config_c1(jmax=97, kmax=69),
            api.config_c2(jmax=129, kmax=41, fsmach=0.4, alfa=2.0, rey=2e6, ds_wall=1e-4),
            api.cmesh_case(97, 33, naca=(0.02, 0.4, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=2, irhsy=-3,
                           ilim=4, ilhs=1, iconstant_cfl=1, dt=20.0, fsmach=0.73, alfa=2.8, rey=6.5e6)]


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
def test_every_tuning_candidate_is_bitwise_the_same(precision):
    cases = _cases()
    ref = _run(precision, cases, (0, 0, 0, 0))
    for c in tune.CANDIDATES:
        out = _run(precision, cases, c)
        for (q, r), (q0, r0) in zip(out, ref):
            assert np.array_equal(q, q0), c
            assert r.cl == r0.cl and r.cd == r0.cd, c
            assert abs(r.rsum_last - r0.rsum_last) <= 1e-13 * r0.rsum_last, c


def test_tuning_table_applies_to_its_class_only():
    """A table entry for this batch's class gives the same bits as the same
    choice set by options; an entry for another class leaves the default."""
    cases = _cases()
    choice = (1, 8, 4, 0)
    by_option = _run(OT2D_FP64, cases, choice)
    by_table = _run(OT2D_FP64, cases, table={(129, 69): choice})
    for (q, _), (q0, _) in zip(by_table, by_option):
        assert np.array_equal(q, q0)
    other = _run(OT2D_FP64, cases, table={(65, 25): (2, 4, 0, 0)})
    default = _run(OT2D_FP64, cases, (0, 0, 0, 1))
    for (q, _), (q0, _) in zip(other, default):
        assert np.array_equal(q, q0)


def test_gpu_tune_one_class_caches_a_candidate(tmp_path):
    import torch
    path = str(tmp_path / "tuning.json")
    gpu = torch.cuda.get_device_name(0)
    choices, timings = tune.tune(tune.gpu_measure_for_class(OT2D_FP32_MIXED, batch=4, iters=3), ((129, 33),), gpu,
                                 OT2D_FP32_MIXED, cache_path=path)
    assert choices[(129, 33)] in tune.CANDIDATES
    assert all(t > 0 for t in timings[(129, 33)].values())
    again, t2 = tune.tune(None, ((129, 33),), gpu, OT2D_FP32_MIXED, cache_path=path, batch=4)
    assert again == choices and t2[(129, 33)] is None
    assert set(json.load(open(path))) == {tune.class_key(gpu, OT2D_FP32_MIXED, 129, 33, 4)}
