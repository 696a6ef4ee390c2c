"""Python host API over libturns2d_gb300.so.

Mirrors the reference's set-up path (read_inputs / set_pointers_globals /
initia, src/setup.f and src/init.f) and exposes the batched solver.  All
compute runs in the native library; this module only marshals arguments.
The library must be built (turns2d_urans_git_gb300.build.build()); there is
no fallback.
"""
import ctypes as C
import os

import numpy as np

from .abi import Inputs, Params, Result, default_inputs, lib_path, OT2D_FP64, OT2D_FP32_MIXED

_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class NativeLibraryMissing(RuntimeError):
    pass


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise NativeLibraryMissing(
                "libturns2d_gb300.so not found at %s; run turns2d_urans_git_gb300.build.build()" % path)
        L = C.CDLL(path)
        L.ot2d_params_from_inputs.argtypes = [C.POINTER(Inputs), C.POINTER(Params)]
        L.ot2d_cmesh_bc_table.argtypes = [C.POINTER(Inputs), C.c_int32]
        L.ot2d_mesh_naca4_cmesh.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
                                            C.c_double, C.c_double, _dp, _dp]
        L.ot2d_solver_create.argtypes = [C.c_int32, C.c_int32]
        L.ot2d_solver_create.restype = C.c_void_p
        L.ot2d_solver_destroy.argtypes = [C.c_void_p]
        L.ot2d_solver_destroy.restype = None
        L.ot2d_solver_set_option.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        L.ot2d_solver_add.argtypes = [C.c_void_p, C.POINTER(Params), _dp, _dp, C.c_double, C.c_int32]
        L.ot2d_solver_iterate.argtypes = [C.c_void_p, C.c_int32]
        L.ot2d_solver_sync.argtypes = [C.c_void_p]
        L.ot2d_solver_live.argtypes = [C.c_void_p]
        L.ot2d_solver_result.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Result)]
        L.ot2d_solver_get_q.argtypes = [C.c_void_p, C.c_int32, _dp]
        L.ot2d_solver_device_bytes.argtypes = [C.c_void_p]
        L.ot2d_solver_device_bytes.restype = C.c_size_t
        L.ot2d_instance_bytes.argtypes = [C.POINTER(Params), C.c_int32]
        L.ot2d_instance_bytes.restype = C.c_size_t
        L.ot2d_solver_queued.argtypes = [C.c_void_p]
        L.ot2d_solver_stream.argtypes = [C.c_void_p]
        L.ot2d_solver_graph_kernels.argtypes = [C.c_void_p]
        L.ot2d_solver_stream.restype = C.c_void_p
        _lib = L
    return _lib


def dptr(a):
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)


def params_from_inputs(inp):
    p = Params()
    rc = lib().ot2d_params_from_inputs(C.byref(inp), C.byref(p))
    if rc != 0:
        raise ValueError("ot2d_params_from_inputs failed (%d)" % rc)
    return p


def naca4_cmesh(jmax, kmax, n_wake, m=0.0, p=0.0, t=0.12, ds_wall=1e-3, r_far=20.0):
    """Vertex grid (xv, yv) of shape (kmax, jmax) in C order == Fortran (jmax,kmax)."""
    xv = np.zeros((kmax, jmax))
    yv = np.zeros((kmax, jmax))
    rc = lib().ot2d_mesh_naca4_cmesh(jmax, kmax, n_wake, m, p, t, ds_wall, r_far, dptr(xv), dptr(yv))
    if rc != 0:
        raise ValueError("mesh generation failed (%d)" % rc)
    return xv, yv


def cmesh_case(jmax, kmax, n_wake=None, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, r_far=20.0, **kw):
    """Inputs + params + grid of one single-C-mesh case.  `kw` are namelist
    overrides (see abi.default_inputs)."""
    if n_wake is None:
        n_wake = (jmax - 1) // 8
    inp = default_inputs(jmax=jmax, kmax=kmax, **kw)
    lib().ot2d_cmesh_bc_table(C.byref(inp), n_wake + 1)
    prm = params_from_inputs(inp)
    xv, yv = naca4_cmesh(jmax, kmax, n_wake, naca[0], naca[1], naca[2], ds_wall, r_far)
    return inp, prm, xv, yv


# ---- the benchmark configurations (inputs of the reference's namelist) ----

def config_c1(jmax=257, kmax=65):
    """Inviscid NACA 0012, M=0.80, alpha=1.25, MUSCL (irhsy=-3, ilim=1),
    LU-SGS, local CFL 10."""
    return cmesh_case(jmax, kmax, naca=(0.0, 0.0, 0.12), ds_wall=1e-3, invisc=1, lamin=1,
                      irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1, dt=10.0, fsmach=0.80, alfa=1.25)


def config_pitching(jmax=129, kmax=33, viscous=False, iturb=1, ntac=2, itnmax=4, dt=0.05, rf=0.2, angmax=2.0,
                    xac=0.25, fsmach=0.5, alfa=0.0, rey=1e6, ds_wall=None):
    """Time-accurate pitching NACA 0012 (iunst=1, motiontype=1: alpha(t) =
    alfa + angmax*(1 - cos(rf*t)) about (xac, 0)): dual time stepping with
    itnmax Newton iterations per physical step dt at order ntac, MUSCL,
    LU-SGS, pseudo-time CFL 1; Euler, or RANS (iturb 1 SA / 2 SST)."""
    kw = dict(invisc=1, lamin=1)
    if viscous:
        kw = dict(invisc=0, lamin=0, iturb=iturb, rey=rey, vnuinf=3.0)
    if ds_wall is None:
        ds_wall = wall_spacing(kmax) if viscous else 1e-3
    return cmesh_case(jmax, kmax, naca=(0.0, 0.0, 0.12), ds_wall=ds_wall, irhsy=-3, ilim=1, ilhs=1,
                      iconstant_cfl=1, idual=1, iunst=1, motiontype=1, ntac=ntac, itnmax=itnmax, dt=dt, rf=rf,
                      angmax=angmax, xac=xac, yac=0.0, fsmach=fsmach, alfa=alfa, **kw)


def config_c2(jmax=513, kmax=129, fsmach=0.15, alfa=10.0, rey=6e6, naca=(0.0, 0.0, 0.12), ds_wall=1e-6):
    """Viscous RANS-SA NACA 0012, M=0.15, alpha=10, Re=6e6, MUSCL, LU-SGS,
    local CFL 50, nu_tilde_inf = 3 nu_inf."""
    return cmesh_case(jmax, kmax, naca=naca, ds_wall=ds_wall, invisc=0, lamin=0, iturb=1,
                      irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1, dt=50.0, fsmach=fsmach, alfa=alfa,
                      rey=rey, vnuinf=3.0)


def config_c3(jmax=769, kmax=193, fsmach=0.73, alfa=2.8, rey=6.5e6, naca=(0.02, 0.4, 0.12), ds_wall=5e-7, dt=2.0,
              ilhs=2):
    """Transonic k-omega SST on a cambered NACA 2412 C-mesh: WENO5
    reconstruction (ilim 4) with Roe fluxes and the diagonalised ADI
    operator (ilhs 2 pentadiagonal, 3 upwind tridiagonal), local time step
    dt (CFL)."""
    return cmesh_case(jmax, kmax, naca=naca, ds_wall=ds_wall, invisc=0, lamin=0, iturb=2, irhsy=-3, ilim=4,
                      ilhs=ilhs, iconstant_cfl=1, dt=dt, fsmach=fsmach, alfa=alfa, rey=rey)


def wall_spacing(kmax, r_far=20.0, ratio=1.2, floor=1e-6):
    """First-cell wall spacing of a C-mesh with kmax points across: the
    spacing whose geometric stretching at `ratio` reaches the far field, but
    not below `floor` (1e-6 chords, y+ < 1 at Re ~ 1e7).  Coarse meshes with
    a 1e-6 spacing would need stretching ratios above 1.3, on which the SA
    solve diverges (the oracle does the same)."""
    return max(floor, r_far * (ratio - 1.0) / (ratio ** (kmax - 1) - 1.0))


def config_c4_sample(rng, sizes=((129, 33), (257, 65), (385, 97), (513, 129), (769, 193))):
    """One seeded batched-SA request: NACA m in U[0,0.06], p in U[0.2,0.6],
    t in U[0.08,0.18]; size from `sizes`; M in U[0.3,0.85], alpha in U[-2,8],
    Re in U[1e6,1e7]."""
    jmax, kmax = sizes[int(rng.integers(len(sizes)))]
    m, pp, t = rng.uniform(0, 0.06), rng.uniform(0.2, 0.6), rng.uniform(0.08, 0.18)
    M, a, Re = rng.uniform(0.3, 0.85), rng.uniform(-2.0, 8.0), rng.uniform(1e6, 1e7)
    return config_c2(jmax, kmax, fsmach=M, alfa=a, rey=Re, naca=(m, pp, t), ds_wall=wall_spacing(kmax))


def config_c5_ts(rng, nspec=None):
    """One time-spectral pitching request on NACA 0012 257x65: N in {3,5,7},
    alpha(t) = alpha0 + 5 deg sin(k t), alpha0 in U[0,10], k in U[0.05,0.15],
    M = 0.3, SA."""
    if nspec is None:
        nspec = int(rng.choice([3, 5, 7]))
    a0, k = rng.uniform(0.0, 10.0), rng.uniform(0.05, 0.15)
    return cmesh_case(257, 65, naca=(0.0, 0.0, 0.12), ds_wall=wall_spacing(65), invisc=0, lamin=0, iturb=1,
                      irhsy=-3, ilim=1, ilhs=1, iconstant_cfl=1, dt=50.0, fsmach=0.3, alfa=a0, rey=6e6,
                      vnuinf=3.0, timespectral=1, nspec=nspec, rf=k, angmax=5.0, xac=0.25, motiontype=1)


# Convergence rule of the FP32-mixed path.  Its f32 residual stops falling
# 2-3 decades below its peak (rounding of O(1) fluxes in the large far-field
# cells), so an 8-10 decade drop of the L2 norm never happens in f32.  A mixed
# solve is converged once the norm is 2 decades below its peak and CL and CD
# stayed within 2e-6 and 4e-7 over 8 samples 200 iterations apart; on cases
# the FP64 path converges 10 decades, the forces so obtained are within
# 1e-6 of FP64's (tests/test_gpu_mixed.py).
MIXED_RULE = {"dcl": 2e-6, "dcd": 4e-7, "every": 200, "decades": 2}


class Solver:
    """Batched device-resident solver (ot2d_solver_*)."""

    def __init__(self, precision=OT2D_FP64, device=0, check_every=25, keep_q=False):
        L = lib()
        self._h = L.ot2d_solver_create(device, precision)
        if not self._h:
            raise RuntimeError("ot2d_solver_create failed (no GPU or bad arguments)")
        L.ot2d_solver_set_option(self._h, 1, int(check_every))
        L.ot2d_solver_set_option(self._h, 2, 1 if keep_q else 0)
        self.precision = precision

    def set_force_tol(self, dcl, dcd, every=0, decades=1):
        """Converge also on stable forces (see ot2d_solver_set_force_tol):
        CL and CD within dcl / dcd over 8 samples taken `every` iterations
        apart (0: one per status check), with the L2 norm `decades` below
        its peak."""
        f = lib().ot2d_solver_set_force_tol
        f.argtypes = [C.c_void_p, C.c_double, C.c_double]
        rc = f(self._h, float(dcl), float(dcd))
        rc = rc or lib().ot2d_solver_set_option(self._h, 3, int(every))
        rc = rc or lib().ot2d_solver_set_option(self._h, 4, int(decades))
        if rc != 0:
            raise RuntimeError("ot2d_solver_set_force_tol failed (%d)" % rc)

    def set_mixed_rule(self):
        """The convergence rule of the FP32-mixed path (MIXED_RULE)."""
        self.set_force_tol(MIXED_RULE["dcl"], MIXED_RULE["dcd"], MIXED_RULE["every"], MIXED_RULE["decades"])

    def close(self):
        if self._h:
            lib().ot2d_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, prm, xv, yv, orders=10.0, max_iters=2000):
        xv = np.ascontiguousarray(xv, dtype=np.float64)
        yv = np.ascontiguousarray(yv, dtype=np.float64)
        rc = lib().ot2d_solver_add(self._h, C.byref(prm), dptr(xv), dptr(yv), float(orders), int(max_iters))
        if rc < 0:
            raise RuntimeError("ot2d_solver_add failed (%d)" % -rc)
        return rc

    def iterate(self, n):
        rc = lib().ot2d_solver_iterate(self._h, int(n))
        if rc != 0:
            raise RuntimeError("ot2d_solver_iterate failed (%d)" % rc)

    def sync(self):
        rc = lib().ot2d_solver_sync(self._h)
        if rc != 0:
            raise RuntimeError("ot2d_solver_sync failed (%d)" % rc)

    def live(self):
        """Submitted requests not yet retired (queued ones included)."""
        return lib().ot2d_solver_live(self._h)

    def queued(self):
        """Submitted requests still waiting for device memory."""
        return lib().ot2d_solver_queued(self._h)

    def result(self, iid):
        r = Result()
        rc = lib().ot2d_solver_result(self._h, int(iid), C.byref(r))
        if rc != 0:
            raise KeyError(iid)
        return r

    def get_q(self, iid, prm):
        q = np.zeros(prm.jd * prm.kd * prm.nspec * prm.nq)
        rc = lib().ot2d_solver_get_q(self._h, int(iid), dptr(q))
        if rc != 0:
            raise RuntimeError("ot2d_solver_get_q failed (%d)" % rc)
        return q

    def device_bytes(self):
        return lib().ot2d_solver_device_bytes(self._h)

    def store(self, iid, directory):
        """Write fort.8 / fort.9 (and SA.dat / komega.dat) of a live instance
        into `directory` (ot2d_solver_store, the astore record layout)."""
        f = lib().ot2d_solver_store
        f.argtypes = [C.c_void_p, C.c_int32, C.c_char_p]
        rc = f(self._h, int(iid), os.fsencode(directory))
        if rc != 0:
            raise RuntimeError("ot2d_solver_store failed (%d)" % rc)

    def store_on_retire(self, iid, directory):
        """Store the instance into `directory` when it retires (None cancels)."""
        f = lib().ot2d_solver_store_on_retire
        f.argtypes = [C.c_void_p, C.c_int32, C.c_char_p]
        rc = f(self._h, int(iid), None if directory is None else os.fsencode(directory))
        if rc != 0:
            raise RuntimeError("ot2d_solver_store_on_retire failed (%d)" % rc)

    def add_restart(self, prm, xv, yv, directory, orders=10.0, max_iters=2000):
        """Admit a solve that starts from `directory`/fort.3 (fort_TS<n>.3)."""
        xv = np.ascontiguousarray(xv, dtype=np.float64)
        yv = np.ascontiguousarray(yv, dtype=np.float64)
        f = lib().ot2d_solver_add_restart
        f.argtypes = [C.c_void_p, C.POINTER(Params), _dp, _dp, C.c_char_p, C.c_double, C.c_int32]
        rc = f(self._h, C.byref(prm), dptr(xv), dptr(yv), os.fsencode(directory), float(orders), int(max_iters))
        if rc < 0:
            raise RuntimeError("ot2d_solver_add_restart failed (%d)" % -rc)
        return rc

    def add_state(self, prm, xv, yv, q, orders=10.0, max_iters=2000):
        """Admit a solve that starts from the state q (jd,kd,nspec,nq in the
        reference layout; q(...,nq) is ignored)."""
        xv = np.ascontiguousarray(xv, dtype=np.float64)
        yv = np.ascontiguousarray(yv, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        if q.size != prm.jd * prm.kd * prm.nspec * prm.nq:
            raise ValueError("q has %d values, expected jd*kd*nspec*nq" % q.size)
        f = lib().ot2d_solver_add_state
        f.argtypes = [C.c_void_p, C.POINTER(Params), _dp, _dp, _dp, C.c_double, C.c_int32]
        rc = f(self._h, C.byref(prm), dptr(xv), dptr(yv), dptr(q), float(orders), int(max_iters))
        if rc < 0:
            raise RuntimeError("ot2d_solver_add_state failed (%d)" % -rc)
        return rc

    def set_log(self, path):
        """Append one JSON line per retired request to `path` (None stops)."""
        f = lib().ot2d_solver_set_log
        f.argtypes = [C.c_void_p, C.c_char_p]
        rc = f(self._h, None if path is None else os.fsencode(path))
        if rc != 0:
            raise RuntimeError("ot2d_solver_set_log failed (%d)" % rc)

    def set_option(self, key, value):
        rc = lib().ot2d_solver_set_option(self._h, int(key), int(value))
        if rc != 0:
            raise RuntimeError("ot2d_solver_set_option(%d, %d) failed (%d)" % (key, value, rc))

    def stream(self):
        return lib().ot2d_solver_stream(self._h)

    def graph_kernels(self):
        """Kernel launches per batched iteration (kernel nodes of the
        iteration's CUDA graph for the current live set)."""
        n = lib().ot2d_solver_graph_kernels(self._h)
        if n < 0:
            raise RuntimeError("ot2d_solver_graph_kernels failed (%d)" % -n)
        return n


def instance_bytes(prm, precision):
    return lib().ot2d_instance_bytes(C.byref(prm), int(precision))
