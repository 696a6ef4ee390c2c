"""Seeded overset grid systems for the interpolation tests: nmesh meshes of
random sizes, a random state (J > 0), and donor / fringe lists in the
layout of the reference's connectivity (src/connectivity.f:2-25): 1-based
indices, Fortran-ordered arrays (idsize, 2, nmesh, nspec) etc."""
import numpy as np

from turns2d_urans_git_gb300.abi import Params


def make_params(nspec=1, iturb=1):
    p = Params()
    p.nspec, p.iturb = nspec, iturb
    p.nmv = 4
    p.nv = 4 + (0, 1, 2)[iturb]
    p.nq = p.nv + 1
    # one mesh's sizes for params_global (do_interpolations takes each
    # mesh's own from jmx, kmx)
    p.nhalo, p.nadd, p.jmax, p.kmax, p.jd, p.kd = 1, 1, 18, 10, 19, 11
    return p


def make_system(p, seed, dims=((19, 11), (14, 9), (23, 7)), ndonor=(17, 9, 21), nfringe=(12, 15, 8), dup=True,
                poly=None):
    """Returns a dict of the reference's arguments.  poly: optional
    f(j, k) -> value that sets q*J (mean flow) and q (turbulence) of every
    mesh to a bi-quadratic field, for exactness checks."""
    rng = np.random.default_rng(seed)
    nm, ns = len(dims), p.nspec
    jmx = np.array([d[0] for d in dims], dtype=np.int32)
    kmx = np.array([d[1] for d in dims], dtype=np.int32)
    blocks = []
    for jm, km in dims:
        q = rng.uniform(0.5, 2.0, (jm, km, ns, p.nq))
        q[..., p.nq - 1] = rng.uniform(0.5, 4.0, (jm, km, ns))
        if poly is not None:
            jj, kk = np.meshgrid(np.arange(1, jm + 1), np.arange(1, km + 1), indexing="ij")
            f = poly(jj, kk)
            for n in range(p.nv):
                if n < p.nmv:
                    q[:, :, :, n] = (f * (n + 1))[:, :, None] / q[..., p.nq - 1]
                else:
                    q[:, :, :, n] = (f * (n + 1))[:, :, None]
        blocks.append(q.ravel(order="F"))
    qg = np.concatenate(blocks)
    idsize = max(max(ndonor), max(nfringe)) + 2
    shp2 = (idsize, 2, nm, ns)
    idonor = np.zeros(shp2, dtype=np.int32, order="F")
    imesh = np.zeros(shp2, dtype=np.int32, order="F")
    frac = np.zeros(shp2, dtype=np.float64, order="F")
    ibc = np.zeros((idsize, nm, ns), dtype=np.int32, order="F")
    nfr = np.zeros((nm, ns), dtype=np.int32, order="F")
    ndo = np.zeros((nm, ns), dtype=np.int32, order="F")
    iis = np.zeros((nm, ns), dtype=np.int32, order="F")
    iie = np.zeros((nm, ns), dtype=np.int32, order="F")
    for s in range(ns):
        ptr = 1
        for im, (jm, km) in enumerate(dims):
            nd = ndonor[im]
            ndo[im, s] = nd
            iis[im, s] = ptr
            iie[im, s] = ptr + nd - 1
            idonor[:nd, 0, im, s] = rng.integers(2, jm, nd)
            idonor[:nd, 1, im, s] = rng.integers(2, km, nd)
            frac[:nd, :, im, s] = rng.uniform(-0.5, 0.5, (nd, 2))
            ptr += nd
        bcdim = ptr - 1
        for im, (jm, km) in enumerate(dims):
            nf = nfringe[im]
            cells = rng.choice(jm * km, size=nf, replace=False)
            imesh[:nf, 0, im, s] = cells % jm + 1
            imesh[:nf, 1, im, s] = cells // jm + 1
            if dup and nf >= 3:   # one cell listed twice: the later entry wins
                imesh[nf - 1, :, im, s] = imesh[0, :, im, s]
            ibc[:nf, im, s] = rng.integers(1, bcdim + 1, nf)
            nfr[im, s] = nf
        iie[nm - 1, s] = bcdim
    return dict(qg=qg, jmx=jmx, kmx=kmx, ibcg=ibc, imeshg=imesh, idonorg=idonor, fracg=frac, nfringeg=nfr,
                ndonorg=ndo, iisptrg=iis, iieptrg=iie, idsize=idsize, qsize=qg.size, nmesh=nm)


def oracle_interp(lib, ptr, p, sysd):
    import ctypes as C
    qg = sysd["qg"].copy()
    lib.oro_do_interpolations(C.byref(p), ptr(qg), ptr(sysd["jmx"]), ptr(sysd["kmx"]), ptr(sysd["ibcg"]),
                              ptr(sysd["imeshg"]), ptr(sysd["idonorg"]), ptr(sysd["fracg"]), ptr(sysd["nfringeg"]),
                              ptr(sysd["ndonorg"]), ptr(sysd["iisptrg"]), ptr(sysd["iieptrg"]), sysd["idsize"],
                              sysd["qsize"], sysd["nmesh"])
    return qg
