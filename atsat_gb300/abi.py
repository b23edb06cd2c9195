"""ctypes mirrors of the structs in include/atsat_dyn.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import fields as F

OK = 0
E_INVALID, E_UNSUPPORTED, E_CUDA, E_TIMEOUT, E_NONFINITE_INPUT, E_NOMEM, E_UNBOUND = (
    -1, -2, -3, -4, -5, -6, -7)
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
                + [("reserved", C.c_int32 * 4)])


class PStats(C.Structure):
    _fields_ = [("sweeps", C.c_int32), ("reserved0", C.c_int32),
                ("src_clamped", C.c_double), ("max_abs_update", C.c_double)]


class PoissonStats(C.Structure):
    _fields_ = [("method", C.c_int32), ("iterations", C.c_int32), ("inner", C.c_int32), ("converged", C.c_int32),
                ("rel_residual", C.c_double), ("ms", C.c_double), ("reserved", C.c_double * 4)]


POISSON_METHODS = ["sor64", "sor32", "refine_sor", "direct64", "direct32", "refine_direct"]


class Diag(C.Structure):
    _fields_ = [("launches", C.c_int64), ("nonfinite", C.c_int64), ("timeout", C.c_int32),
                ("reserved", C.c_int32 * 5)]


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
