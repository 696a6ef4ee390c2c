"""Test cases: seeded C-meshes and physical states, set up by the oracle
(initia, src/init.f:2-177), shared by the CPU and GPU tests."""
import ctypes as C

import numpy as np

from tests import oracle_binding as ob
from turns2d_urans_git_gb300 import api


class Case:
    """All arrays of one single-instance (nspec=1) case in reference layout."""

    def __init__(self, jmax=65, kmax=25, viscous=False, ilim=1, irhsy=-3, seed=0, naca=(0.0, 0.0, 0.12),
                 perturb=0.02, alfa=2.0, fsmach=0.5, rey=1e6, ds_wall=None, n_wake=None, istep0=10, iturb=1):
        if ds_wall is None:
            ds_wall = 2e-3 if not viscous else 1e-4
        kw = dict(irhsy=irhsy, ilim=ilim, ilhs=1, iconstant_cfl=1, fsmach=fsmach, alfa=alfa)
        if viscous:
            kw.update(invisc=0, lamin=0, iturb=iturb, dt=50.0, rey=rey, vnuinf=3.0)
        else:
            kw.update(invisc=1, lamin=1, dt=10.0)
        self.inp, _, xv, yv = api.cmesh_case(jmax, kmax, n_wake=n_wake, naca=naca, ds_wall=ds_wall, **kw)
        self.p = ob.read_inputs(self.inp)
        self.p.istep0 = istep0
        p = self.p
        self.jd, self.kd = p.jd, p.kd
        n2 = p.jd * p.kd
        self.n2 = n2
        self.xv = np.ascontiguousarray(xv.ravel())
        self.yv = np.ascontiguousarray(yv.ravel())
        L = ob.lib()
        z = lambda: np.zeros(n2)
        self.x, self.y, self.xx, self.xy, self.yx, self.yy = z(), z(), z(), z(), z(), z()
        self.ug, self.vg, self.turmu, self.tscale, self.bt = z(), z(), z(), z(), z()
        self.ugv = np.zeros(p.jmax * p.kmax)
        self.vgv = np.zeros(p.jmax * p.kmax)
        self.iblank = np.ones(n2, dtype=np.int32)
        self.q = np.zeros(n2 * p.nq)
        self.s = np.zeros(n2 * p.nv)
        pp = C.byref(p)
        L.oro_find_cellcenter(pp, ob.ptr(self.x), ob.ptr(self.y), ob.ptr(self.xv), ob.ptr(self.yv))
        nneg = L.oro_metfv(pp, ob.ptr(self.q), ob.ptr(self.xv), ob.ptr(self.yv), ob.ptr(self.xx), ob.ptr(self.xy),
                           ob.ptr(self.yx), ob.ptr(self.yy))
        assert nneg == 0
        L.oro_qzero(pp, ob.ptr(self.q))
        L.oro_qdivj(pp, ob.ptr(self.q))
        if perturb:
            self.perturb(seed, perturb)

    def perturb(self, seed, amp):
        """Random but physical state: density, velocity and pressure of every
        cell perturbed by O(amp) relative to freestream."""
        rng = np.random.default_rng(seed)
        p, n2 = self.p, self.n2
        q = self.q.reshape(p.nq, n2)
        J = q[p.nq - 1]
        rho = q[0] * J * (1.0 + amp * rng.uniform(-1, 1, n2))
        u = q[1] / q[0] + amp * rng.uniform(-1, 1, n2)
        v = q[2] / q[0] + amp * rng.uniform(-1, 1, n2)
        pres = p.pinf * (1.0 + amp * rng.uniform(-1, 1, n2))
        e = pres / p.gm1 + 0.5 * rho * (u * u + v * v)
        q[0] = rho / J
        q[1] = rho * u / J
        q[2] = rho * v / J
        q[3] = e / J
        if not p.lamin and p.iturb == 1:
            q[4] = p.vnuinf * (1.0 + 50.0 * rng.uniform(0, 1, n2))
            self.turmu[:] = 0.1 * rng.uniform(0, 1, n2)
        elif not p.lamin and p.iturb == 2:
            # k and omega (times rho) spread over decades around freestream
            q[4] = rho * p.tkeinf * 10.0 ** rng.uniform(0, 3, n2)
            q[5] = rho * p.tomegainf * 10.0 ** rng.uniform(0, 3, n2)
            self.turmu[:] = 0.1 * rng.uniform(0, 1, n2)
        self.tscale[:] = 0.0

    def copy(self):
        import copy
        c = copy.copy(self)
        for k, v in list(self.__dict__.items()):
            if isinstance(v, np.ndarray):
                setattr(c, k, v.copy())
        return c


def relerr(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), floor)
    return float(np.max(np.abs(a - b)) / scale)
