"""ctypes binding of the CPU FP64 oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: the oracle is the checker, never the thing
measured or shipped.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs load it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from turns2d_urans_git_gb300.abi import Params, Inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
# the -O3 build the benchmark times (never a parity checker)
ORACLE_FAST_SO = os.path.join(ORACLE_DIR, "liboracle_fast.so")

_lib = None
_lib_fast = None

_P = C.POINTER(Params)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def build():
    subprocess.run(["make", "-s", "-j2", "-C", ORACLE_DIR], check=True)


def lib():
    """The checker build of the oracle."""
    global _lib
    if _lib is None:
        _lib = _load(ORACLE_SO)
    return _lib


def lib_fast():
    """The -O3 build of the same sources, timed as the CPU baseline."""
    global _lib_fast
    if _lib_fast is None:
        _lib_fast = _load(ORACLE_FAST_SO)
    return _lib_fast


def _load(path):
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.oro_read_inputs.argtypes = [C.POINTER(Inputs), _P]
    L.oro_find_cellcenter.argtypes = [_P, _dp, _dp, _dp, _dp]
    L.oro_metfv.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    L.oro_metfv.restype = C.c_int
    L.oro_qzero.argtypes = [_P, _dp]
    L.oro_qdivj.argtypes = [_P, _dp]
    L.oro_computeTScoefs.argtypes = [C.c_int, _dp]
    L.oro_timespectralrhs.argtypes = [_P, _dp, _dp, _dp, C.c_int]
    L.oro_find_coord_TS_orig.argtypes = [_P, _dp, _dp, _dp, _dp, C.c_double]
    L.oro_find_timemetrics_TS_orig.argtypes = [_P, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp, _dp, _dp]
    L.oro_bc.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    L.oro_rbc.argtypes = [_P, _dp, _dp]
    L.oro_rhsup.argtypes = [_P, _dp, _dp, _dp, _dp, _ip, _dp, _dp]
    L.oro_visrhs.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    L.oro_time_step.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    L.oro_ilu2d.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    L.oro_preilu2d.argtypes = [_P] + [_dp] * 11
    L.oro_rhslom.argtypes = [_P, _dp, _dp, _dp]
    L.oro_vmu_sa.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    L.oro_vmu_sa.restype = C.c_double
    L.oro_komegasst.argtypes = [_P] + [_dp] * 14 + [_ip, _dp]
    L.oro_arc2d.argtypes = [_P] + [_dp] * 9 + [_ip, _dp, _dp]
    L.oro_arc2d_precon.argtypes = [_P] + [_dp] * 9 + [_ip, _dp, _dp]
    L.oro_do_interpolations.argtypes = [_P, _dp, _ip, _ip, _ip, _ip, _ip, _dp, _ip, _ip, _ip, _ip, C.c_int32,
                                         C.c_int64, C.c_int32]
    L.oro_monitor.argtypes = [_P, _dp]
    L.oro_monitor.restype = C.c_int
    L.oro_force2d.argtypes = [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    L.oro_step.argtypes = [_P] + [_dp] * 6 + [_ip] + [_dp] * 12 + [_dp, _ip]
    L.oro_step_u.argtypes = [_P] + [_dp] * 6 + [_ip] + [_dp] * 12 + [_dp, _ip] + [_dp] * 5
    L.oro_step_u.restype = C.c_int
    L.oro_step.restype = C.c_int
    L.oro_solve.argtypes = [_P, _dp, _dp, C.c_int, C.c_double, _dp, _dp, _dp]
    L.oro_solve.restype = C.c_int
    L.oro_solve_from.argtypes = [_P, _dp, _dp, C.c_int, C.c_double, _dp, C.c_int, _dp, _dp, _dp]
    L.oro_solve_from.restype = C.c_int
    return L


def ptr(a):
    """ctypes pointer to a numpy array's data (must be contiguous)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    raise TypeError(a.dtype)


def read_inputs(inp):
    p = Params()
    lib().oro_read_inputs(C.byref(inp), C.byref(p))
    return p


def solve(p, xv, yv, nsteps, orders=0.0, fast=False):
    """Run the oracle driver; returns (iterations, hist[it, nsp], forces[nsp,5], q).
    fast: the -O3 timing build instead of the checker."""
    nsp = p.nspec
    hist = np.zeros((nsteps, nsp))
    forces = np.zeros((nsp, 5))
    q = np.zeros(p.jd * p.kd * nsp * p.nq)
    n = (lib_fast() if fast else lib()).oro_solve(C.byref(p), ptr(np.ascontiguousarray(xv, dtype=np.float64)),
                        ptr(np.ascontiguousarray(yv, dtype=np.float64)), nsteps, orders,
                        ptr(hist), ptr(forces), ptr(q))
    return n, hist[:abs(n)], forces, q


def solve_from(p, xv, yv, nsteps, q_init, istep0, orders=0.0):
    """The oracle driver from a restart state q_init (q(1:nv) / J, flat
    (jd,kd,nspec,nv) or the full (jd,kd,nspec,nq) array) continuing at istep0."""
    nsp = p.nspec
    hist = np.zeros((nsteps, nsp))
    forces = np.zeros((nsp, 5))
    q = np.zeros(p.jd * p.kd * nsp * p.nq)
    qi = np.ascontiguousarray(q_init, dtype=np.float64)
    n = lib().oro_solve_from(C.byref(p), ptr(np.ascontiguousarray(xv, dtype=np.float64)),
                             ptr(np.ascontiguousarray(yv, dtype=np.float64)), nsteps, orders, ptr(qi), int(istep0),
                             ptr(hist), ptr(forces), ptr(q))
    return n, hist[:abs(n)], forces, q


_io = None


def oracle_io():
    """The numpy restatement of the solution / restart files (oracle/oracle_io.py)."""
    global _io
    if _io is None:
        import importlib.util
        path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "oracle_io.py")
        spec = importlib.util.spec_from_file_location("oracle_io", path)
        _io = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(_io)
    return _io


_cases = None


def oracle_cases():
    """The numpy restatement of the benchmark cases (oracle/oracle_cases.py):
    meshes and &bcinp tables built without the product library."""
    global _cases
    if _cases is None:
        import importlib.util
        path = os.path.join(ORACLE_DIR, "oracle_cases.py")
        spec = importlib.util.spec_from_file_location("oracle_cases", path)
        _cases = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(_cases)
    return _cases

