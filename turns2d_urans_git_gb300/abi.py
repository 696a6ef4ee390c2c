"""ctypes mirror of include/ot2d_params.h and include/ot2d.h.

The structures below are byte-for-byte the C structs the library takes; the
field order is the header's.  They mirror the reference's module
`params_global` (src/modules.f:4-213) and the namelist `&inputs`
(src/modules.f:197-208).
"""
import ctypes as C
import os

MAXBC = 25

OT2D_OK = 0
OT2D_ERR_ARG = 1
OT2D_ERR_NORM = 2
OT2D_ERR_MONITOR = 3
OT2D_ERR_CUDA = 4
OT2D_ERR_NOPARAMS = 5
OT2D_ERR_NOMEM = 6
OT2D_ERR_TIMEOUT = 7

OT2D_ERR_IO = 8

OT2D_FP64 = 0
OT2D_FP32_MIXED = 1

# solver options (ot2d_solver_set_option)
OT2D_OPT_CHECK_EVERY = 1
OT2D_OPT_KEEP_Q = 2
OT2D_OPT_FORCE_EVERY = 3
OT2D_OPT_FORCE_DECADES = 4
OT2D_OPT_POLL_LIMIT = 5
OT2D_OPT_BUDGET_MB = 6
OT2D_OPT_LU_LAG = 7
OT2D_OPT_LU_GROUP = 8
OT2D_OPT_RT_SHAPE = 9
OT2D_OPT_PIPELINE = 10

_I = C.c_int32
_D = C.c_double


class Params(C.Structure):
    _fields_ = [(n, _I) for n in (
        "jmax", "kmax", "jd", "kd", "nhalo", "nadd", "jbeg", "jend", "kbeg", "kend",
        "jtail1", "jtail2", "jle", "half", "nq", "nv", "nmv", "nturb", "nspec",
        "irhsy", "ilim", "ilhs", "iconstant_cfl", "idual", "idual_turb",
        "iunst", "ntac", "itnmax", "iread",
        "invisc", "lamin", "iturb", "itrans", "timespectral", "iprecon", "motiontype",
        "istep", "istep0", "itn", "npnorm")] + [(n, _D) for n in (
        "gamma", "gm1", "ggm1", "pr", "rey", "tinf", "rmue", "fsmach", "fmtip", "alfa",
        "rinf", "uinf", "vinf", "einf", "pinf", "htinf", "ainf", "vnuinf", "tkeinf", "tomegainf",
        "epse", "dt", "h", "timeac", "dualtime", "cfltur",
        "rotf", "rf", "angmax", "xac", "yac", "Mp", "totime", "theta_col")] + [
        ("nbc", _I), ("pad0", _I),
        ("ibtyp", _I * MAXBC), ("ibdir", _I * MAXBC), ("jbcs", _I * MAXBC), ("jbce", _I * MAXBC),
        ("kbcs", _I * MAXBC), ("kbce", _I * MAXBC)]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


class Inputs(C.Structure):
    _fields_ = [(n, _I) for n in (
        "jmax", "kmax", "nhalo", "jtail1", "half", "invisc", "lamin", "iturb", "itrans",
        "irhsy", "ilim", "ilhs", "iconstant_cfl", "idual", "idual_turb",
        "iunst", "ntac", "itnmax", "iread", "timespectral", "nspec", "motiontype", "npnorm")] + [
        (n, _D) for n in ("fsmach", "fmtip", "alfa", "rey", "vnuinf", "tuinf", "dt", "timeac", "epse", "cfltur",
                          "rf", "angmax", "xac", "yac")] + [
        ("nbc", _I), ("pad0", _I),
        ("ibtyp", _I * MAXBC), ("ibdir", _I * MAXBC), ("jbcs", _I * MAXBC), ("jbce", _I * MAXBC),
        ("kbcs", _I * MAXBC), ("kbce", _I * MAXBC)]


class Tuning(C.Structure):
    """ot2d_tuning: launch choices for batches of one mesh-size class."""
    _fields_ = [("kd_max", _I), ("jd_max", _I), ("rt_shape", _I), ("lu_group", _I), ("lu_lag", _I),
                ("pipeline", _I)]


class Result(C.Structure):
    _fields_ = [("id", _I), ("status", _I), ("iterations", _I), ("converged", _I),
                ("rsum_first", _D), ("rsum_last", _D), ("cl", _D), ("cd", _D), ("cm", _D), ("cpower", _D),
                ("t_admit", _D), ("t_done", _D), ("t_submit", _D)]


def default_inputs(**kw):
    """Namelist defaults of the reference (src/modules.f:170-190) with
    keyword overrides."""
    i = Inputs()
    i.jmax, i.kmax, i.nhalo, i.jtail1, i.half = 109, 36, 1, 19, 0
    i.invisc, i.lamin, i.iturb, i.itrans = 1, 1, 1, 0
    i.irhsy, i.ilim, i.ilhs, i.iconstant_cfl, i.idual, i.idual_turb = -3, 0, 1, 0, 0, 0
    i.iunst, i.ntac, i.itnmax, i.iread = 0, 1, 1, 0
    i.timespectral, i.nspec, i.motiontype, i.npnorm = 0, 1, 1, 25
    i.fsmach, i.fmtip, i.alfa, i.rey, i.vnuinf, i.tuinf = 0.16, 0.0, 0.0, 3900000.0, 0.1, 0.2
    i.dt, i.timeac, i.epse, i.cfltur = 0.1, 1.0, 0.01, 1.0
    i.rf, i.angmax, i.xac, i.yac = 0.0, 0.0, 0.0, 0.0
    for k, v in kw.items():
        if not hasattr(i, k):
            raise KeyError(k)
        setattr(i, k, v)
    return i


def lib_path():
    here = os.path.dirname(os.path.abspath(__file__))
    return os.path.join(here, "libturns2d_gb300.so")
