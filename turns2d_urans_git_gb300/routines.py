"""The reference's hot-path subroutines, by their reference names.

Each function forwards to the drop-in C-ABI routine that replaces the
Fortran subroutine of the same name (declared in include/ot2d.h) with the
reference's argument order.  Arrays are flat float64 / int32 buffers in the
reference's column-major layout: numpy arrays (host memory, copied in and
out by the library) or CUDA tensors / any object exposing
``data_ptr()`` (device memory, used in place).  Scalars are passed by
reference as the Fortran callers do.  A non-zero status raises
``RoutineError``.
"""
import ctypes as C

import numpy as np

from .abi import Params
from .api import lib

_i = C.c_int32


class RoutineError(RuntimeError):
    def __init__(self, name, code):
        super().__init__("%s returned status %d" % (name, code))
        self.code = code


def _p(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if not (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]):
            raise ValueError("arrays must be contiguous")
        if a.dtype not in (np.float64, np.int32):
            raise TypeError("arrays must be float64 or int32, got %s" % a.dtype)
        return C.c_void_p(a.ctypes.data)
    raise TypeError(type(a))


def _ref(v):
    return C.byref(_i(int(v)))


def _call(name, *args):
    f = getattr(lib(), name)
    f.restype = C.c_int
    rc = f(*args)
    if rc != 0:
        raise RoutineError(name, rc)
    return rc


def set_params(p: Params):
    """params_global of the current mesh (replaces set_pointers_globals)."""
    _call("ot2d_set_params", C.byref(p))


def rhsup(q, s, xx, xy, yx, yy, x, y, xv, yv, xold, yold, xole, yole, iblank, ugv, vgv, jd, kd, nei, im, bt):
    """src/eulerrhs.f:2 -- s -= inviscid flux differences."""
    _call("ot2d_rhsup", _p(q), _p(s), _p(xx), _p(xy), _p(yx), _p(yy), _p(x), _p(y), _p(xv), _p(yv), _p(xold),
          _p(yold), _p(xole), _p(yole), _p(iblank), _p(ugv), _p(vgv), _ref(jd), _ref(kd), _ref(nei), _ref(im), _p(bt))


def visrhs(turmu, q, s, xx, xy, yx, yy, ug, vg, tscale, iblank, jd, kd):
    """src/visrhs.f:2 -- s += viscous flux differences."""
    _call("ot2d_visrhs", _p(turmu), _p(q), _p(s), _p(xx), _p(xy), _p(yx), _p(yy), _p(ug), _p(vg), _p(tscale),
          _p(iblank), _ref(jd), _ref(kd))


def bc(q, x, y, xx, xy, yx, yy, ug, vg, im, jd, kd, bt):
    """src/bc.f:2 -- halo cells of q."""
    _call("ot2d_bc", _p(q), _p(x), _p(y), _p(xx), _p(xy), _p(yx), _p(yy), _p(ug), _p(vg), _ref(im), _ref(jd),
          _ref(kd), _p(bt))


def rbc(q, s, x, y, xx, xy, yx, yy, ug, vg, im, jd, kd, bt):
    """src/bc.f:88 -- halo cells of the residual."""
    _call("ot2d_rbc", _p(q), _p(s), _p(x), _p(y), _p(xx), _p(xy), _p(yx), _p(yy), _p(ug), _p(vg), _ref(im),
          _ref(jd), _ref(kd), _p(bt))


def time_step(q, xx, xy, yx, yy, ug, vg, tscale, bt, iblank, jd, kd):
    """src/time.f:2 -- local time step."""
    _call("ot2d_time_step", _p(q), _p(xx), _p(xy), _p(yx), _p(yy), _p(ug), _p(vg), _p(tscale), _p(bt), _p(iblank),
          _ref(jd), _ref(kd))


def ilu2d(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, tscale):
    """src/lhs.f:470 -- LU-SGS implicit operator (s already times tscale)."""
    _call("ot2d_ilu2d", _p(q), _p(s), _ref(jd), _ref(kd), _ref(js), _ref(je), _ref(ks), _ref(ke), _p(xx), _p(xy),
          _p(yx), _p(yy), _p(ug), _p(vg), _p(turmu), _p(tscale))


def preilu2d(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, tscale, bt):
    """src/lhs.f:2 -- LU-SGS with Turkel's low-Mach preconditioner (bt of time_step)."""
    _call("ot2d_preilu2d", _p(q), _p(s), _ref(jd), _ref(kd), _ref(js), _ref(je), _ref(ks), _ref(ke), _p(xx), _p(xy),
          _p(yx), _p(yy), _p(ug), _p(vg), _p(turmu), _p(tscale), _p(bt))


def rhslom(q, s, jd, kd, js, je, ks, ke, bt):
    """src/sources.f:97 -- the interior residual times the low-Mach preconditioner."""
    _call("ot2d_rhslom", _p(q), _p(s), _ref(jd), _ref(kd), _ref(js), _ref(je), _ref(ks), _ref(ke), _p(bt))


def arc2d(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, iblank, tscale, bt):
    """src/lhs.f:817 -- diagonalised ADI (pentadiagonal line inversions)."""
    _call("ot2d_arc2d", _p(q), _p(s), _ref(jd), _ref(kd), _ref(js), _ref(je), _ref(ks), _ref(ke), _p(xx), _p(xy),
          _p(yx), _p(yy), _p(ug), _p(vg), _p(turmu), _p(iblank), _p(tscale), _p(bt))


def arc2d_precon(q, s, jd, kd, js, je, ks, ke, xx, xy, yx, yy, ug, vg, turmu, iblank, tscale, bt):
    """src/lhs.f:1060 -- the ADI operator with Turkel's low-Mach preconditioner."""
    _call("ot2d_arc2d_precon", _p(q), _p(s), _ref(jd), _ref(kd), _ref(js), _ref(je), _ref(ks), _ref(ke), _p(xx),
          _p(xy), _p(yx), _p(yy), _p(ug), _p(vg), _p(turmu), _p(iblank), _p(tscale), _p(bt))


def do_interpolations(qg, jmx, kmx, ibcg, imeshg, idonorg, fracg, nfringeg, ndonorg, iisptrg, iieptrg, idsize,
                      qsize, nmesh):
    """src/connectivity.f:2 -- overset interpolation: donors gathered, fringe cells overwritten."""
    _call("ot2d_do_interpolations", _p(qg), _p(jmx), _p(kmx), _p(ibcg), _p(imeshg), _p(idonorg), _p(fracg),
          _p(nfringeg), _p(ndonorg), _p(iisptrg), _p(iieptrg), _ref(idsize), _ref(qsize), _ref(nmesh))


def vmu_sa(q, s, turmu, x, y, xv, yv, xx, xy, yx, yy, ug, vg, jd, kd, tscale, iblank, im, nsp):
    """src/samodel2d.f:2 -- one Spalart-Allmaras update of q(:,:,5) and turmu."""
    _call("ot2d_vmu_sa", _p(q), _p(s), _p(turmu), _p(x), _p(y), _p(xv), _p(yv), _p(xx), _p(xy), _p(yx), _p(yy),
          _p(ug), _p(vg), _ref(jd), _ref(kd), _p(tscale), _p(iblank), _ref(im), _ref(nsp))


def komegasst(q, s, turmu, x, y, xv, yv, xx, xy, yx, yy, ug, vg, jd, kd, tscale, iblank, im):
    """src/komegasst.f:2 -- one k-omega SST update of q(:,:,5:6) and turmu."""
    _call("ot2d_komegasst", _p(q), _p(s), _p(turmu), _p(x), _p(y), _p(xv), _p(yv), _p(xx), _p(xy), _p(yx), _p(yy),
          _p(ug), _p(vg), _ref(jd), _ref(kd), _p(tscale), _p(iblank), _ref(im))


def timespectralrhs(q, s, Ds, jd, kd, nsp):
    """src/sources.f:2 -- time-spectral coupling term of instance nsp."""
    _call("ot2d_timespectralrhs", _p(q), _p(s), _p(Ds), _ref(jd), _ref(kd), _ref(nsp))


def step(q, qtn, qtnm1, qnewt, s, x, y, xv, yv, iblank, xx, xy, yx, yy, ug, vg, ugv, vgv, xold, yold, xole, yole,
         turmu, tscale, bt, Ds, im, jd, kd):
    """src/step.f:2 -- one iteration of every time instance; returns the
    (rsum, resrho, resmax) norms of each instance."""
    f = lib().ot2d_step
    f.restype = C.c_int
    rc = f(_p(q), _p(qtn), _p(qtnm1), _p(qnewt), _p(s), _p(x), _p(y), _p(xv), _p(yv), _p(iblank), _p(xx), _p(xy),
           _p(yx), _p(yy), _p(ug), _p(vg), _p(ugv), _p(vgv), _p(xold), _p(yold), _p(xole), _p(yole), _p(turmu),
           _p(tscale), _p(bt), _p(Ds), _ref(im), _ref(jd), _ref(kd))
    norms = last_norms(64)
    if rc != 0:
        raise RoutineError("ot2d_step", rc)
    return norms


def last_norms(n):
    out = np.zeros(3 * n)
    lib().ot2d_last_norms(C.c_void_p(out.ctypes.data), 3 * n)
    return out


def monitor(q, jd, kd):
    """src/step.f:332 -- returns mstop (1 on a non-positive a^2 or NaN)."""
    mstop = _i(0)
    _call("ot2d_monitor", C.byref(mstop), _p(q), _ref(jd), _ref(kd))
    return mstop.value


def force2d(jd, kd, x, y, xv, yv, q, xx, xy, yx, yy, nsp=1):
    """src/forces.f:130 -- (cfx, cfy, cm0, cpower)."""
    out = [C.c_double(0) for _ in range(4)]
    _call("ot2d_force2d", _ref(jd), _ref(kd), _p(x), _p(y), _p(xv), _p(yv), _p(q), _p(xx), _p(xy), _p(yx), _p(yy),
          C.byref(out[0]), C.byref(out[1]), C.byref(out[2]), C.byref(out[3]), _ref(nsp))
    return tuple(o.value for o in out)


def find_cellcenter(x, y, xv, yv, jd, kd, im=1):
    """src/setup.f:111."""
    _call("ot2d_find_cellcenter", _p(x), _p(y), _p(xv), _p(yv), _ref(jd), _ref(kd), _ref(im))


def metfv(q, x, y, xv, yv, xx, xy, yx, yy, jd, kd, im=1):
    """src/setup.f:440 -- J into q(:,:,nq) and the J-scaled metrics."""
    _call("ot2d_metfv", _p(q), _p(x), _p(y), _p(xv), _p(yv), _p(xx), _p(xy), _p(yx), _p(yy), _ref(jd), _ref(kd),
          _ref(im))


# ---- solution / restart files (src/io.f, src/init.f) ----------------------
# Fortran unit numbers refer to the library's own unit table: open them with
# unit_open() where the reference has `open(unit=...)`.

def unit_open(unit, path, formatted=False, for_write=True):
    """open(unit, file=path, form='formatted'|'unformatted')."""
    f = lib().ot2d_unit_open
    f.argtypes = [_i, C.c_char_p, _i, _i]
    _call("ot2d_unit_open", _i(unit), str(path).encode(), _i(1 if formatted else 0), _i(1 if for_write else 0))


def unit_close(unit):
    _call("ot2d_unit_close", _i(unit))


def unit_write_ints(unit, values):
    v = np.ascontiguousarray(values, dtype=np.int32)
    _call("ot2d_unit_write_ints", _i(unit), C.c_void_p(v.ctypes.data), _i(v.size))


def unit_read_ints(unit, n):
    v = np.zeros(n, dtype=np.int32)
    _call("ot2d_unit_read_ints", _i(unit), C.c_void_p(v.ctypes.data), _i(n))
    return v


def astore(x, y, iblank, q, iturb, itrans, jgmx, kgmx, nmesh, ipointer, igrd, iqdim, istep0, ts, nspec):
    """src/io.f:2 -- writes the solution files into the current directory;
    returns the (jd, kd) of the last mesh."""
    jd, kd = _i(0), _i(0)
    jg = np.ascontiguousarray(jgmx, dtype=np.int32)
    kg = np.ascontiguousarray(kgmx, dtype=np.int32)
    ip = np.asfortranarray(np.asarray(ipointer, dtype=np.int32).reshape(nmesh, 5, order="F"))
    _call("ot2d_astore", _p(x), _p(y), _p(iblank), _p(q), _ref(iturb), _ref(itrans), _p(jg), _p(kg), _ref(nmesh),
          C.c_void_p(ip.ctypes.data), _ref(igrd), _ref(iqdim), C.byref(jd), C.byref(kd), _ref(istep0),
          _ref(1 if ts else 0), _ref(nspec))
    return jd.value, kd.value


def store(q, x, y, iblank, jd, kd, lg, lq):
    """src/io.f:278 (lg, lq: one unit per time instance)."""
    lg = np.ascontiguousarray(lg, dtype=np.int32)
    lq = np.ascontiguousarray(lq, dtype=np.int32)
    _call("ot2d_store", _p(q), _p(x), _p(y), _p(iblank), _ref(jd), _ref(kd), _p(lg), _p(lq))


def storevnu(x, y, iblank, q, jd, kd, lq, ltur):
    """src/io.f:173."""
    lq = np.ascontiguousarray(lq, dtype=np.int32)
    lt = np.ascontiguousarray(ltur, dtype=np.int32)
    _call("ot2d_storevnu", _p(x), _p(y), _p(iblank), _p(q), _ref(jd), _ref(kd), _p(lq), _p(lt))


def storekomega(x, y, iblank, q, jd, kd, lq, ltur):
    """src/io.f:218."""
    lq = np.ascontiguousarray(lq, dtype=np.int32)
    lt = np.ascontiguousarray(ltur, dtype=np.int32)
    _call("ot2d_storekomega", _p(x), _p(y), _p(iblank), _p(q), _ref(jd), _ref(kd), _p(lq), _p(lt))


def grid(xv, yv, iblank, jd, kd, logg):
    """src/io.f:343."""
    _call("ot2d_grid", _p(xv), _p(yv), _p(iblank), _ref(jd), _ref(kd), _ref(logg))


def restr2(q, jd, kd, logq):
    """src/io.f:383 (q: one time instance, q(jd,kd,nq))."""
    _call("ot2d_restr2", _p(q), _ref(jd), _ref(kd), _ref(logq))


def restr_turb(q, jd, kd, logq):
    """src/io.f:408."""
    _call("ot2d_restr_turb", _p(q), _ref(jd), _ref(kd), _ref(logq))


def qdivj(q, jd, kd):
    """src/init.f:180."""
    _call("ot2d_qdivj", _p(q), _ref(jd), _ref(kd))


# ---- time-accurate pieces (src/motion.f, src/time.f) -------------------------

def pitch(x, y, xv, yv, xold, yold, xole, yole, ug, vg, jd, kd, init=0):
    """src/motion.f:546 -- step params.istep of the pitching motion."""
    _call("ot2d_pitch", _ref(init), _p(x), _p(y), _p(xv), _p(yv), _p(xold), _p(yold), _p(xole), _p(yole), _p(ug),
          _p(vg), _ref(jd), _ref(kd))


def stqol(q, qtn, qtnm1, qnewt, jd, kd):
    """src/time.f:110."""
    _call("ot2d_stqol", _p(q), _p(qtn), _p(qtnm1), _p(qnewt), _ref(jd), _ref(kd))
