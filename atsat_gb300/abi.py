"""ctypes mirrors of the structs in include/atsat_dyn.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import fields as F

OK = 0
E_INVALID, E_UNSUPPORTED, E_CUDA, E_TIMEOUT, E_NONFINITE_INPUT, E_NOMEM, E_UNBOUND, E_TOO_LARGE = (
    -1, -2, -3, -4, -5, -6, -7, -8)
FP64, MIXED = 0, 1

K_RK_STAGE, K_LEVEL_MEAN, K_METRIC_SCAN, K_PRESS_SOURCE, K_PRESS_SWEEP, K_PRESS_BOUNDARY, \
    K_GLUE, K_RHS = range(8)
K_NAMES = ["rk_stage", "level_mean", "metric_scan", "press_source", "press_sweep",
           "press_boundary", "glue", "rhs", "prepare"]


class Grid(C.Structure):
    _fields_ = [("im", C.c_int32), ("jm", C.c_int32), ("km", C.c_int32), ("reserved0", C.c_int32),
                ("rad_z", C.POINTER(C.c_double)), ("the_z", C.POINTER(C.c_double)),
                ("dr", C.c_double), ("dthe", C.c_double), ("dphi", C.c_double)]


class Params(C.Structure):
    _fields_ = ([(n, C.c_double) for n, _ in F.PARAM_DOUBLES]
                + [(n, C.c_int32) for n, _ in F.PARAM_INTS]
                + [("reserved", C.c_int32 * 3)])


class TurbParams(C.Structure):
    """atsat_dyn_turb_params: the knobs and constants of Turbulence<cSaturnModel>::run."""
    _fields_ = [("model", C.c_int32), ("turb_free", C.c_int32), ("clamp_pass", C.c_int32), ("abl_taper", C.c_int32),
                ("curv", C.c_int32), ("buoy", C.c_int32), ("k_bg", C.c_double), ("l_bg", C.c_double),
                ("nue_max_phys", C.c_double), ("vel_star_max", C.c_double), ("vel_star_ref", C.c_double),
                ("z_0", C.c_double), ("nue_gas", C.c_double), ("abl_height", C.c_double),
                ("ep", C.c_double * 3), ("lv", C.c_double * 3), ("ls", C.c_double * 3), ("t_0", C.c_double * 3),
                ("reserved", C.c_double * 4)]


TURB_K_EPSILON, TURB_K_OMEGA, TURB_K_OMEGA_SST = 0, 1, 2

# the reference's defaults (Turbulence.h:119-187, 348-352, 712-713, 812-813; the moist gases' constants of
# cSaturnModel.h read back from its build: H2O, NH3, CH4)
TURB_DEFAULTS = dict(model=TURB_K_OMEGA_SST, turb_free=1, clamp_pass=1, abl_taper=0, curv=1, buoy=3, k_bg=1.0,
                     l_bg=0.0, nue_max_phys=1.0e5, vel_star_max=0.002 ** 0.5 * 200.0, vel_star_ref=0.4, z_0=0.1,
                     nue_gas=1.8e-5, abl_height=20000.0, ep=(8.1253, 7.6752, 7.6752),
                     lv=(2.5009e6, 1.372e6, 5.11e5), ls=(2.8339e6, 1.832e6, 5.11e5), t_0=(273.15, 195.5, 90.69))


def make_turb_params(**over) -> TurbParams:
    d = dict(TURB_DEFAULTS)
    for k, v in over.items():
        if k not in d:
            raise KeyError(k)
        d[k] = v
    tp = TurbParams()
    for k, v in d.items():
        if isinstance(v, tuple):
            getattr(tp, k)[:] = v
        else:
            setattr(tp, k, v)
    return tp


class PStats(C.Structure):
    _fields_ = [("sweeps", C.c_int32), ("reserved0", C.c_int32),
                ("src_clamped", C.c_double), ("max_abs_update", C.c_double)]


class PoissonStats(C.Structure):
    _fields_ = [("method", C.c_int32), ("iterations", C.c_int32), ("inner", C.c_int32), ("converged", C.c_int32),
                ("rel_residual", C.c_double), ("ms", C.c_double), ("sweeps_per_pass", C.c_int32), ("pad", C.c_int32),
                ("sweep_ms", C.c_double), ("reserved", C.c_double * 2)]


POISSON_METHODS = ["sor64", "sor32", "refine_sor", "direct64", "direct32", "refine_direct"]


class Diag(C.Structure):
    _fields_ = [("launches", C.c_int64), ("nonfinite", C.c_int64), ("timeout", C.c_int32),
                ("tuned_from_cache", C.c_int32), ("reserved", C.c_int32 * 4)]


# ChemistrySat::ThermalPropertiesSat of the default composition (planet/ChemistrySat.h:475-530),
# as the reference computes them (read back from the reference build, bit for bit).
CP_MIX = float.fromhex("0x1.3a544e8a8f013p+13")    # 10058.538350217079 J/(kg K)
R_MIX_RHO = 1.382                                   # r_mix, kg/m3
R_MIX_GAS = float.fromhex("0x1.6ba7dd06e410fp+11")  # R_mix, 2909.245730824892 J/(kg K)


def default_params(**over) -> dict:
    d = {n: v for n, v in F.PARAM_DOUBLES}
    d.update({n: v for n, v in F.PARAM_INTS})
    d["cp_mix"] = CP_MIX
    d["r_mix"] = R_MIX_RHO
    d["R_mix"] = R_MIX_GAS
    for k, v in over.items():
        if k not in d:
            raise KeyError(k)
        d[k] = v
    return d


def make_params(d: dict) -> Params:
    p = Params()
    for n, _ in F.PARAM_DOUBLES:
        setattr(p, n, float(d[n]))
    for n, _ in F.PARAM_INTS:
        setattr(p, n, int(d[n]))
    return p


class GridHold:
    """A Grid struct plus the numpy arrays it points into (kept alive together)."""

    def __init__(self, grid):
        self.rad_z = np.ascontiguousarray(grid.rad_z, dtype=np.float64)
        self.the_z = np.ascontiguousarray(grid.the_z, dtype=np.float64)
        self.s = Grid(grid.im, grid.jm, grid.km, 0,
                      self.rad_z.ctypes.data_as(C.POINTER(C.c_double)),
                      self.the_z.ctypes.data_as(C.POINTER(C.c_double)),
                      grid.dr, grid.dthe, grid.dphi)


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))
