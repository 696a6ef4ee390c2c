"""CPU tests of the solution / restart file layer: the oracle's files read
back with scipy.io.FortranFile (an independent reader and writer of Fortran
sequential unformatted records), the Tecplot edit descriptors, and the
library's unit-table record routines (no CUDA involved).  No GPU needed."""
import os

import numpy as np
import pytest

from tests import oracle_binding as ob
from turns2d_urans_git_gb300 import api
from turns2d_urans_git_gb300.abi import Params

FortranFile = pytest.importorskip("scipy.io").FortranFile


def make_params(iturb, nspec=1, jd=9, kd=7):
    p = Params()
    p.fsmach, p.alfa, p.rey, p.totime = 0.73, 2.5, 6.5e6 / 0.73, 0.125
    p.iturb, p.itrans, p.nspec = iturb, 0, nspec
    p.nv = 4 + (0, 1, 2)[iturb]
    p.nq = p.nv + 1
    p.jd, p.kd, p.jmax, p.kmax, p.nhalo, p.nadd = jd, kd, jd - 1, kd - 1, 1, 1
    return p


def make_mesh(p, jd, kd, seed, ragged_iblank=False):
    rng = np.random.default_rng(seed)
    n = jd * kd * p.nspec
    q = rng.uniform(-2.0, 2.0, n * p.nq)
    q[(p.nq - 1) * n:] = rng.uniform(0.5, 4.0, n)             # J > 0
    q[4 * n:p.nv * n] = np.abs(q[4 * n:p.nv * n]) + 0.1           # turbulence variables > 0
    q[:n] = np.abs(q[:n]) + 0.1                                   # density > 0 (SST divides by it)
    ib = rng.integers(0, 2, n).astype(np.int32) if ragged_iblank else np.ones(n, dtype=np.int32)
    return dict(q=q, x=rng.uniform(-30, 30, n), y=rng.uniform(-30, 30, n), iblank=ib, jd=jd, kd=kd)


@pytest.mark.parametrize("iturb,nspec,nmesh", [(0, 1, 1), (1, 1, 1), (2, 1, 1), (1, 3, 1), (0, 1, 2), (2, 2, 2)])
def test_oracle_astore_records_read_by_scipy(tmp_path, iturb, nspec, nmesh):
    """Every record of the oracle's fort.8 / fort.9 is where io.f:2-170 puts
    it, as an independent Fortran-record reader sees it."""
    oio = ob.oracle_io()
    p = make_params(iturb, nspec)
    dims = [(9, 7), (6, 5)][:nmesh]
    meshes = [make_mesh(p, j, k, 10 + i, ragged_iblank=nmesh > 1) for i, (j, k) in enumerate(dims)]
    q0 = [m["q"].copy() for m in meshes]
    oio.astore(str(tmp_path), p, meshes, istep0=1234, ts=nspec > 1)
    for s in range(nspec):
        fq = FortranFile(oio.sol_file(str(tmp_path), nspec > 1, s + 1, "q", iturb), "r")
        fg = FortranFile(oio.sol_file(str(tmp_path), nspec > 1, s + 1, "g", iturb), "r")
        for f in (fq, fg):
            if nmesh > 1:
                assert list(f.read_ints(np.int32)) == [nmesh]
            assert list(f.read_ints(np.int32)) == [v for d in dims for v in d]
        for (jd, kd), m, qa in zip(dims, meshes, q0):
            n2 = jd * kd
            q = qa.reshape((jd, kd, nspec, p.nq), order="F")
            hdr = fq.read_reals(np.float64)
            assert list(hdr) == [p.fsmach, p.alfa, p.rey * p.fsmach, p.totime]
            Q = fq.read_reals(np.float64).reshape((jd, kd, 4), order="F")
            J = q[:, :, s, p.nq - 1]
            for n in range(4):
                assert np.array_equal(Q[:, :, n], q[:, :, s, n] * J)
            if iturb:
                T = fq.read_reals(np.float64).reshape((jd, kd, p.nv - 4), order="F")
                assert np.array_equal(T, q[:, :, s, 4:p.nv])
            if nmesh > 1:
                x, y, ib = fg.read_record(np.dtype(("<f8", n2)), np.dtype(("<f8", n2)), np.dtype(("<i4", n2)))
                assert np.array_equal(ib, m["iblank"].reshape((n2, nspec), order="F")[:, s])
            else:
                xy = fg.read_reals(np.float64)
                x, y = xy[:n2], xy[n2:]
            assert np.array_equal(x, m["x"].reshape((n2, nspec), order="F")[:, s])
            assert np.array_equal(y, m["y"].reshape((n2, nspec), order="F")[:, s])
        if iturb == 2:
            for (jd, kd), qa in zip(dims, q0):
                T = fq.read_reals(np.float64)   # storekomega's second copy
                assert np.array_equal(T, qa.reshape((jd * kd, nspec, p.nq), order="F")[:, s, 4:p.nv].ravel(order="F"))
        assert list(fq.read_ints(np.int32)) == [1234]
        with pytest.raises(Exception):
            fq.read_ints(np.int32)
        fq.close(); fg.close()
    # store's round trip leaves q(1:4) at (q*J)/J
    for m, qa in zip(meshes, q0):
        n = m["jd"] * m["kd"] * nspec
        J = qa[(p.nq - 1) * n:]
        for v in range(4):
            assert np.array_equal(m["q"][v * n:(v + 1) * n], (qa[v * n:(v + 1) * n] * J) / J)


@pytest.mark.parametrize("iturb", [0, 1, 2])
def test_oracle_restart_reads_scipy_written_file(tmp_path, iturb):
    """init.f:138-170 on a fort.3 written by scipy.io.FortranFile."""
    oio = ob.oracle_io()
    p = make_params(iturb)
    jd, kd, n2 = p.jd, p.kd, p.jd * p.kd
    rng = np.random.default_rng(5)
    Q = rng.uniform(0.5, 2.0, (jd, kd, 4))
    T = rng.uniform(0.5, 2.0, (jd, kd, p.nv - 4))
    f = FortranFile(str(tmp_path / "fort.3"), "w")
    f.write_record(np.array([jd, kd], dtype=np.int32))
    f.write_record(np.array([0.5, 1.0, 2e6, 3.25]))
    f.write_record(np.asfortranarray(Q).ravel(order="F"))
    if iturb:
        f.write_record(np.asfortranarray(T).ravel(order="F"))
    f.write_record(np.array([77], dtype=np.int32))
    f.close()
    q = np.zeros(n2 * p.nq)
    J = rng.uniform(0.5, 4.0, n2)
    q[(p.nq - 1) * n2:] = J
    totime, istep0 = oio.restart(str(tmp_path), p, q, jd, kd, ts=False)
    assert totime == 3.25 and istep0 == 77
    qq = q.reshape((n2, p.nq), order="F")
    for n in range(4):
        assert np.array_equal(qq[:, n], Q[:, :, n].ravel(order="F") / J)
    if iturb:
        assert np.array_equal(qq[:, 4:p.nv], T.reshape((n2, p.nv - 4), order="F"))


def test_oracle_tecplot_edit_descriptors():
    oio = ob.oracle_io()
    assert oio.fmt_f(1.5) == "       1.5000000000000"
    assert oio.fmt_f(-0.25) == "      -0.2500000000000"
    assert oio.fmt_f(1234567.0) == " 1234567.0000000000000"
    assert oio.fmt_f(12345678.0) == "12345678.0000000000000"
    assert oio.fmt_f(-12345678.0) == "*" * 22         # does not fit F22.13
    assert oio.fmt_f(123456789.0) == "*" * 22
    assert oio.fmt_f(float("nan")) == " " * 19 + "NaN"
    txt = oio.tec_reals(np.arange(7, dtype=np.float64))
    lines = txt.splitlines()
    assert [len(l) for l in lines] == [66, 66, 22]
    assert oio.tec_ints(np.array([1, 0, 1, 1], dtype=np.int32)) == "         1         0         1\n         1\n"
    assert oio.tec_zone(9, 7) == " ZONE\n I =            9, J =            7\n ZONETYPE = Ordered, DATAPACKING = BLOCK\n"


def test_library_unit_records(tmp_path):
    """ot2d_unit_* frame records exactly as scipy.io.FortranFile does, both
    ways, and a short record is an error (OT2D_ERR_IO = 8)."""
    L = api.lib()
    import ctypes as C
    path = str(tmp_path / "u.bin")
    v = np.array([3, -7, 11], dtype=np.int32)
    assert L.ot2d_unit_open(41, path.encode(), 0, 1) == 0
    assert L.ot2d_unit_write_ints(41, C.c_void_p(v.ctypes.data), 3) == 0
    assert L.ot2d_unit_write_ints(41, C.c_void_p(v.ctypes.data), 1) == 0
    assert L.ot2d_unit_close(41) == 0
    f = FortranFile(path, "r")
    assert list(f.read_ints(np.int32)) == [3, -7, 11]
    assert list(f.read_ints(np.int32)) == [3]
    f.close()
    f = FortranFile(path, "w")
    f.write_record(np.array([5, 6, 7, 8], dtype=np.int32))
    f.write_record(np.array([9], dtype=np.int32))
    f.close()
    out = np.zeros(4, dtype=np.int32)
    assert L.ot2d_unit_open(42, path.encode(), 0, 0) == 0
    assert L.ot2d_unit_read_ints(42, C.c_void_p(out.ctypes.data), 2) == 0   # first items of a longer record
    assert list(out[:2]) == [5, 6]
    assert L.ot2d_unit_read_ints(42, C.c_void_p(out.ctypes.data), 2) == 8   # record shorter than asked
    assert L.ot2d_unit_close(42) == 0
    assert L.ot2d_unit_read_ints(42, C.c_void_p(out.ctypes.data), 1) == 8   # unit not connected
    assert L.ot2d_unit_open(43, str(tmp_path / "missing" / "x").encode(), 0, 0) == 8
