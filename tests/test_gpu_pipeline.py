"""The pipelined iteration (OT2D_OPT_PIPELINE): a batch of 16 or more time
instances runs as two halves on two streams, each half starting an
iteration when the other half's residual is done.  Every request computes
exactly what it computes in the single-graph iteration, bit for bit, in
FP64 and in the FP32-mixed path, through the device-resident and the
host-buffer paths, with requests retiring mid-way."""
import ctypes as C

import numpy as np
import pytest

from turns2d_urans_git_gb300 import api
from turns2d_urans_git_gb300.abi import OT2D_FP32_MIXED, OT2D_FP64, OT2D_OPT_PIPELINE

pytestmark = pytest.mark.gpu


def _cases(n=20):
    rng = np.random.default_rng(5)
    out = []
    for i in range(n):
        jm, km = ((65, 25), (97, 33), (129, 33), (97, 69))[i % 4]
        if i % 5 == 4:
            out.append(api.config_c1(jmax=jm, kmax=km))
        else:
            out.append(api.config_c2(jmax=jm, kmax=km, fsmach=float(rng.uniform(0.3, 0.6)),
                                     alfa=float(rng.uniform(-2, 6)), rey=2e6, ds_wall=1e-4))
    # a time-spectral request (three coupled instances stay in one half)
    out.append(api.cmesh_case(97, 33, ds_wall=1e-3, invisc=0, lamin=0, iturb=1, irhsy=-3, ilim=1, ilhs=1,
                              iconstant_cfl=1, dt=20.0, fsmach=0.3, alfa=2.0, rey=2e6, vnuinf=3.0, timespectral=1,
                              nspec=3, rf=0.1, angmax=5.0, xac=0.25, motiontype=1))
    return out


def _run(precision, pipeline, cases, caps):
    sv = api.Solver(precision, check_every=9, keep_q=True)
    sv.set_option(OT2D_OPT_PIPELINE, pipeline)
    ids = [sv.add(c[1], c[2], c[3], orders=0.0, max_iters=m) for c, m in zip(cases, caps)]
    while sv.live() > 0:
        sv.iterate(7)
    sv.sync()
    out = [(sv.get_q(i, c[1]), sv.result(i)) for i, c in zip(ids, cases)]
    sv.close()
    return out


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
@pytest.mark.parametrize("pipe", [1, 2])
def test_pipelined_iteration_is_bitwise_the_single_graph(precision, pipe):
    """Two pipelined halves (1) or four independent parts (2) against one
    graph (0), requests retiring at different iterations."""
    cases = _cases()
    caps = [30 + 3 * (i % 7) for i in range(len(cases))]   # requests retire at different iterations
    a = _run(precision, 0, cases, caps)
    b = _run(precision, pipe, cases, caps)
    for (qa, ra), (qb, rb), m in zip(a, b, caps):
        assert ra.status == rb.status == 0 and ra.iterations == rb.iterations == m
        assert np.array_equal(qa, qb)
        assert ra.rsum_last == rb.rsum_last and ra.cl == rb.cl and ra.cd == rb.cd


def test_pipelined_host_buffer_path_matches():
    """ot2d_solver_iterate_host over a pipelined batch: the uploads and
    downloads see both halves' work."""
    cases = _cases(18)[:18]
    steps = 6
    qs = {}
    for pipe in (0, 1):
        sv = api.Solver(OT2D_FP32_MIXED, check_every=100, keep_q=True)
        sv.set_option(OT2D_OPT_PIPELINE, pipe)
        ids = [sv.add(c[1], c[2], c[3], orders=0.0, max_iters=1000) for c in cases]
        qh = [np.ascontiguousarray(sv.get_q(i, c[1])) for i, c in zip(ids, cases)]
        ptrs = (C.POINTER(C.c_double) * len(qh))(*[q.ctypes.data_as(C.POINTER(C.c_double)) for q in qh])
        idarr = (C.c_int32 * len(ids))(*ids)
        L = api.lib()
        L.ot2d_solver_iterate_host.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                               C.POINTER(C.POINTER(C.c_double)), C.c_int32]
        assert L.ot2d_solver_iterate_host(sv._h, len(ids), idarr, ptrs, steps) == 0
        qs[pipe] = [q.copy() for q in qh]
        sv.close()
    for qa, qb in zip(qs[0], qs[1]):
        assert np.array_equal(qa, qb)


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
@pytest.mark.parametrize("pipeline", [0, 1, 2])
def test_graph_iteration_is_bitwise_the_sequential_phase_order(precision, pipeline):
    """The captured iteration runs the turbulence solve on a second stream,
    beside the LU-SGS sweeps (and, in the mixed path, its first part beside
    the LU-SGS records as well).  ot2d_solver_profile runs the same
    iterations one phase after the other in step.f's order (residual, rbc,
    ilu2d, turbulence, update) on one stream; both give the same bits, so
    the branches share no data that one writes while the other reads."""
    cases = _cases(18)
    n = 12
    sv = api.Solver(precision, check_every=10 ** 6, keep_q=True)
    sv.set_option(OT2D_OPT_PIPELINE, pipeline)
    ids = [sv.add(c[1], c[2], c[3], orders=0.0, max_iters=10 ** 6) for c in cases]
    sv.iterate(n)
    sv.sync()
    graph = [sv.get_q(i, c[1]) for i, c in zip(ids, cases)]
    sv.close()
    sv = api.Solver(precision, check_every=10 ** 6, keep_q=True)
    ids = [sv.add(c[1], c[2], c[3], orders=0.0, max_iters=10 ** 6) for c in cases]
    L = api.lib()
    L.ot2d_solver_profile.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int32]
    ms = (C.c_double * 7)()
    assert L.ot2d_solver_profile(sv._h, n, ms, 7) == 0
    sv.sync()
    seq = [sv.get_q(i, c[1]) for i, c in zip(ids, cases)]
    sv.close()
    for a, b in zip(graph, seq):
        assert np.array_equal(a, b)


def _host_iterate(sv, ids, cases, steps):
    qh = [np.ascontiguousarray(sv.get_q(i, cases[k][1])) for k, i in ids]
    ptrs = (C.POINTER(C.c_double) * len(qh))(*[q.ctypes.data_as(C.POINTER(C.c_double)) for q in qh])
    idarr = (C.c_int32 * len(ids))(*[i for _, i in ids])
    L = api.lib()
    L.ot2d_solver_iterate_host.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                                           C.POINTER(C.POINTER(C.c_double)), C.c_int32]
    assert L.ot2d_solver_iterate_host(sv._h, len(ids), idarr, ptrs, steps) == 0
    return qh


@pytest.mark.parametrize("precision", [OT2D_FP64, OT2D_FP32_MIXED])
@pytest.mark.parametrize("retire", [0, 3, 8])
def test_host_buffer_path_equals_device_path(precision, retire):
    """ot2d_solver_iterate_host on a batch of 23 time instances (20
    requests of one, one of three) runs it in four parts, each with its own
    graph and stream, so that some parts' copies overlap the others'
    iterations.  Listed requests end with the bits of the device-resident
    iterations (their host buffers and the device state alike).  `retire`
    unlisted requests stop after 3 iterations: with 3 the batch keeps its
    parts, with 8 it falls to 15 instances, below the parts' size, and the
    call finishes in the single graph."""
    cases = _cases(20)          # 20 single-instance requests + one of 3 time instances
    steps = 8
    short = set(range(retire))  # unlisted requests capped at 3 iterations
    out = {}
    for path in ("device", "host"):
        sv = api.Solver(precision, check_every=1, keep_q=True)
        ids = [sv.add(c[1], c[2], c[3], orders=0.0, max_iters=3 if k in short else 1000)
               for k, c in enumerate(cases)]
        listed = [(k, i) for k, i in enumerate(ids) if k not in short]
        if path == "device":
            sv.iterate(steps)
            sv.sync()
            host = None
        else:
            host = _host_iterate(sv, listed, cases, steps)
            sv.sync()
        out[path] = ([sv.get_q(i, cases[k][1]) for k, i in listed], host)
        for k, i in enumerate(ids):
            r = sv.result(i)
            assert r.status == 0 and (k not in short or r.iterations == 3)
        sv.close()
    dev, _ = out["device"]
    hq, hb = out["host"]
    for a, b, c in zip(dev, hq, hb):
        assert np.array_equal(a, b) and np.array_equal(a, c)
