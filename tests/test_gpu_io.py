"""GPU tests of the solution / restart files (src/io.f, src/init.f:138-206)
through the C-ABI: the drop-in astore / store / storevnu / storekomega /
grid / restr2 / restr_turb / qdivj and the batched solver's snapshot,
store-on-retire and restart admission, each against the numpy oracle
(oracle/oracle_io.py) byte for byte, and a stored-and-resumed solve against
the oracle driver continuing from the same restart file.

Tolerance: files and states are bit-exact (the device conversions are single
IEEE multiplies and divides); the resumed FP64 solve agrees with the oracle
to 1e-12 relative, as every FP64 solver test does."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from tests import oracle_binding as ob
from tests.helpers import relerr
from tests.test_io_cpu import make_mesh, make_params
from turns2d_urans_git_gb300 import api, routines as rt
from turns2d_urans_git_gb300.abi import OT2D_FP64, OT2D_FP32_MIXED

pytestmark = pytest.mark.gpu
FortranFile = pytest.importorskip("scipy.io").FortranFile


def _same_files(da, db, names):
    for n in names:
        a = open(os.path.join(da, n), "rb").read()
        b = open(os.path.join(db, n), "rb").read()
        assert a == b, n


def _names(iturb, nspec):
    ts = nspec > 1
    out = []
    for s in range(1, nspec + 1):
        out += ["fort_TS%d.8" % s, "fort_TS%d.9" % s] if ts else ["fort.8", "fort.9"]
        if iturb in (1, 2):
            base = "komega" if iturb == 2 else "SA"
            out.append(("%s_TS%d.dat" % (base, s)) if ts else base + ".dat")
    return out


@pytest.mark.parametrize("iturb,nspec,nmesh", [(0, 1, 1), (1, 1, 1), (2, 1, 1), (1, 3, 1), (0, 1, 2), (2, 2, 2)])
def test_astore_dropin_matches_oracle(tmp_path, monkeypatch, iturb, nspec, nmesh):
    oio = ob.oracle_io()
    p = make_params(iturb, nspec)
    dims = [(9, 7), (6, 5)][:nmesh]
    meshes = [make_mesh(p, j, k, 20 + i, ragged_iblank=nmesh > 1) for i, (j, k) in enumerate(dims)]
    # the reference's packed arrays: meshes one after another, 1-based offsets
    x = np.concatenate([m["x"] for m in meshes])
    y = np.concatenate([m["y"] for m in meshes])
    ib = np.concatenate([m["iblank"] for m in meshes])
    q = np.concatenate([m["q"] for m in meshes])
    ig = np.cumsum([1] + [j * k * nspec for j, k in dims])[:nmesh]
    igq = np.cumsum([1] + [j * k * nspec * p.nq for j, k in dims])[:nmesh]
    ipointer = np.zeros((nmesh, 5), dtype=np.int32, order="F")
    ipointer[:, 0], ipointer[:, 1] = ig, igq
    do = tmp_path / "oracle"
    dl = tmp_path / "lib"
    do.mkdir(); dl.mkdir()
    oio.astore(str(do), p, meshes, istep0=321, ts=nspec > 1)
    rt.set_params(p)
    monkeypatch.chdir(dl)
    jd, kd = rt.astore(x, y, ib, q, iturb, 0, [d[0] for d in dims], [d[1] for d in dims], nmesh, ipointer,
                       x.size, q.size, 321, nspec > 1, nspec)
    assert (jd, kd) == dims[-1]
    _same_files(str(do), str(dl), _names(iturb, nspec))
    # q went through store's (q*J)/J round trip on the device, as the oracle's did
    assert np.array_equal(q, np.concatenate([m["q"] for m in meshes]))


@pytest.mark.parametrize("iturb", [1, 2])
def test_unit_dropins_store_and_restart(tmp_path, monkeypatch, iturb):
    """store + storevnu / storekomega on units opened through the library
    give astore's files; restr2 + restr_turb + qdivj read them back as
    init.f does; grid reads a vertex-grid record."""
    oio = ob.oracle_io()
    p = make_params(iturb)
    m = make_mesh(p, p.jd, p.kd, 31)
    mo = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in m.items()}
    oio.astore(str(tmp_path), p, [mo], istep0=9, ts=False)
    dl = tmp_path / "lib"
    dl.mkdir()
    rt.set_params(p)
    rt.unit_open(1009, dl / "fort.9")
    rt.unit_open(1008, dl / "fort.8")
    rt.unit_write_ints(1009, [p.jd, p.kd])
    rt.unit_write_ints(1008, [p.jd, p.kd])
    q = m["q"]
    rt.store(q, m["x"], m["y"], m["iblank"], p.jd, p.kd, [1009], [1008])
    # astore writes the title lines itself (io.f:100-101, :136-138); the
    # unit-level routine writes the zone
    rt.unit_open(1010, dl / "zone.dat", formatted=True)
    (rt.storekomega if iturb == 2 else rt.storevnu)(m["x"], m["y"], m["iblank"], q, p.jd, p.kd, [1008], [1010])
    rt.unit_write_ints(1008, [9])
    for u in (1008, 1009, 1010):
        rt.unit_close(u)
    tec = dl / ("komega.dat" if iturb == 2 else "SA.dat")
    tec.write_text(oio.tec_title(iturb) + (dl / "zone.dat").read_text())
    _same_files(str(tmp_path), str(dl), _names(iturb, 1))
    assert np.array_equal(q, mo["q"])
    # restart: fort.8 read back as fort.3 through restr2 / restr_turb / qdivj
    shutil.copy(dl / "fort.8", dl / "fort.3")
    n2 = p.jd * p.kd
    qr = np.zeros(n2 * p.nq)
    qr[(p.nq - 1) * n2:] = q[(p.nq - 1) * n2:]
    rt.unit_open(3, dl / "fort.3", for_write=False)
    assert list(rt.unit_read_ints(3, 2)) == [p.jd, p.kd]
    rt.restr2(qr, p.jd, p.kd, 3)
    rt.restr_turb(qr, p.jd, p.kd, 3)
    i0 = rt.unit_read_ints(3, 1)[0]
    rt.unit_close(3)
    rt.qdivj(qr, p.jd, p.kd)
    qo = np.zeros(n2 * p.nq)
    qo[(p.nq - 1) * n2:] = q[(p.nq - 1) * n2:]
    shutil.copy(dl / "fort.8", tmp_path / "fort.3")
    totime, i0o = oio.restart(str(tmp_path), p, qo, p.jd, p.kd, ts=False)
    assert i0 == i0o and totime == p.totime
    assert np.array_equal(qr, qo)
    # grid: one record of xv, yv (jmax, kmax)
    rng = np.random.default_rng(3)
    xv0, yv0 = rng.uniform(-1, 1, p.jmax * p.kmax), rng.uniform(-1, 1, p.jmax * p.kmax)
    f = FortranFile(str(dl / "fort.1"), "w")
    f.write_record(np.array([p.jmax, p.kmax], dtype=np.int32))
    f.write_record(np.concatenate([xv0, yv0]))
    f.close()
    xv, yv, ibg = np.zeros_like(xv0), np.zeros_like(yv0), np.zeros(n2, dtype=np.int32)
    rt.unit_open(1, dl / "fort.1", for_write=False)
    assert list(rt.unit_read_ints(1, 2)) == [p.jmax, p.kmax]
    rt.grid(xv, yv, ibg, p.jd, p.kd, 1)
    rt.unit_close(1)
    assert np.array_equal(xv, xv0) and np.array_equal(yv, yv0) and np.all(ibg == 1)


def _case(kind):
    if kind == "sa":
        _, prm, xv, yv = api.cmesh_case(97, 33, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=1,
                                        irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1, dt=20.0, fsmach=0.5, alfa=3.0,
                                        rey=3e6, vnuinf=3.0)
    elif kind == "sst":
        _, prm, xv, yv = api.cmesh_case(97, 33, naca=(0.02, 0.4, 0.12), ds_wall=1e-3, invisc=0, lamin=0, iturb=2,
                                        irhsy=-3, ilim=4, ilhs=1, iconstant_cfl=1, dt=20.0, fsmach=0.73, alfa=2.8,
                                        rey=6.5e6)
    else:
        _, prm, xv, yv = api.config_c1(jmax=97, kmax=25)
    prm.istep0 = 0
    return prm, xv, yv


def _oracle_mesh(prm, xv, yv, q):
    n2 = prm.jd * prm.kd
    x, y = np.zeros(n2), np.zeros(n2)
    ob.lib().oro_find_cellcenter(C.byref(prm), ob.ptr(x), ob.ptr(y), ob.ptr(np.ascontiguousarray(xv.ravel())),
                                 ob.ptr(np.ascontiguousarray(yv.ravel())))
    return dict(q=q, x=x, y=y, iblank=np.ones(n2, dtype=np.int32), jd=prm.jd, kd=prm.kd)


# FP64 solver-vs-oracle tolerance of each model (the SST source terms call
# pow / exp, which may differ by an ulp between the device and the host)
SOLVE_TOL = {"sa": 1e-12, "sst": 1e-10, "euler": 1e-12}


@pytest.mark.parametrize("kind", ["sa", "sst"])
def test_solver_store_and_resume_fp64(tmp_path, kind):
    """Snapshot a served FP64 instance after N iterations and restart a new
    instance from that file for M more.  The files equal the oracle's astore
    of the instance's state byte for byte and the state after the snapshot
    is the oracle's round trip of it; the resumed state agrees with the
    oracle driver resumed from the same file (iread = 1) to the FP64 solver
    tolerance."""
    oio = ob.oracle_io()
    prm, xv, yv = _case(kind)
    N, M = 15, 10
    do, dl, dr = tmp_path / "o", tmp_path / "l", tmp_path / "r"
    for d in (do, dl, dr):
        d.mkdir()
    sv = api.Solver(OT2D_FP64, check_every=1000)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=1000)
    sv.iterate(N)
    q_before = sv.get_q(iid, prm)
    sv.store(iid, str(dl))
    q_after = sv.get_q(iid, prm)
    q_ostore = q_before.copy()
    oio.astore(str(do), prm, [_oracle_mesh(prm, xv, yv, q_ostore)], istep0=N, ts=False)
    _same_files(str(do), str(dl), _names(prm.iturb, 1))
    assert np.array_equal(q_after, q_ostore)
    n, _, _, q_o = ob.solve(prm, xv.ravel(), yv.ravel(), N)
    assert n == N and relerr(q_before, q_o) <= SOLVE_TOL[kind]
    # resume from the library's file, on both sides
    shutil.copy(dl / "fort.8", dr / "fort.3")
    rid = sv.add_restart(prm, xv, yv, str(dr), orders=0.0, max_iters=1000)
    sv.iterate(M)
    q_r = sv.get_q(rid, prm)
    sv.close()
    n2 = prm.jd * prm.kd
    q_init = np.zeros(n2 * prm.nq)
    q_init[(prm.nq - 1) * n2:] = q_before[(prm.nq - 1) * n2:]
    totime, istep0 = oio.restart(str(dr), prm, q_init, prm.jd, prm.kd, ts=False)
    assert np.array_equal(q_init[:prm.nv * n2], q_after[:prm.nv * n2])
    pr = type(prm).from_buffer_copy(prm)
    pr.iread = 1
    n, _, _, q_ro = ob.solve_from(pr, xv.ravel(), yv.ravel(), M, q_init, istep0)
    assert n == M
    assert relerr(q_r, q_ro) <= SOLVE_TOL[kind]


def test_solver_store_on_retire(tmp_path):
    """An instance stores itself when it reaches its iteration cap, before
    its memory is freed: the files are the oracle's astore of its final
    state (kept with keep_q), istep0 = the iterations run."""
    oio = ob.oracle_io()
    prm, xv, yv = _case("euler")
    dl, do = tmp_path / "l", tmp_path / "o"
    dl.mkdir(); do.mkdir()
    sv = api.Solver(OT2D_FP64, check_every=10, keep_q=True)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=20)
    sv.store_on_retire(iid, str(dl))
    sv.iterate(40)
    assert sv.live() == 0
    r = sv.result(iid)
    assert r.iterations == 20
    q_kept = sv.get_q(iid, prm)          # state after the store's round trip
    sv.close()
    f = FortranFile(str(dl / "fort.8"), "r")
    f.read_ints(np.int32); f.read_reals(np.float64)
    Q = f.read_reals(np.float64)
    assert list(f.read_ints(np.int32)) == [20]
    f.close()
    n2 = prm.jd * prm.kd
    J = q_kept[(prm.nq - 1) * n2:]
    for v in range(4):
        assert np.array_equal(q_kept[v * n2:(v + 1) * n2], Q[v * n2:(v + 1) * n2] / J)
    # the oracle's files from the state the library's record came from
    q_o = q_kept.copy()
    for v in range(4):
        q_o[v * n2:(v + 1) * n2] = Q[v * n2:(v + 1) * n2] / J
    qq = q_o.copy()
    oio.astore(str(do), prm, [_oracle_mesh(prm, xv, yv, qq)], istep0=20, ts=False)
    _same_files(str(do), str(dl), _names(prm.iturb, 1)[1:])
    rec_o = oio.read_records(str(do / "fort.8"))
    rec_l = oio.read_records(str(dl / "fort.8"))
    assert rec_o[0] == rec_l[0] and rec_o[1] == rec_l[1] and rec_o[-1] == rec_l[-1]


def test_solver_mixed_snapshot_and_restart(tmp_path):
    """An FP32-mixed snapshot writes the FP64 master state it holds (Q = q*J)
    and a restart from it restores that state exactly."""
    prm, xv, yv = _case("euler")
    dm, dr = tmp_path / "m", tmp_path / "r"
    dm.mkdir(); dr.mkdir()
    sv = api.Solver(OT2D_FP32_MIXED, check_every=1000)
    iid = sv.add(prm, xv, yv, orders=0.0, max_iters=1000)
    sv.iterate(30)
    q0 = sv.get_q(iid, prm)
    sv.store(iid, str(dm))
    q1 = sv.get_q(iid, prm)
    n2 = prm.jd * prm.kd
    J = q0[(prm.nq - 1) * n2:]
    f = FortranFile(str(dm / "fort.8"), "r")
    assert list(f.read_ints(np.int32)) == [prm.jd, prm.kd]
    f.read_reals(np.float64)
    Q = f.read_reals(np.float64)
    f.close()
    for v in range(4):
        assert np.array_equal(Q[v * n2:(v + 1) * n2], q0[v * n2:(v + 1) * n2] * J)
        assert np.array_equal(q1[v * n2:(v + 1) * n2], Q[v * n2:(v + 1) * n2] / J)
    shutil.copy(dm / "fort.8", dr / "fort.3")
    rid = sv.add_restart(prm, xv, yv, str(dr), orders=0.0, max_iters=1000)
    assert np.array_equal(sv.get_q(rid, prm)[:4 * n2], q1[:4 * n2])
    sv.iterate(5)
    assert sv.result(rid).status == 0
    sv.close()
