"""ORACLE -- TEST INFRASTRUCTURE ONLY: ctypes wrapper of oracle/atsat_oracle.c.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker of the CUDA
path; the product never imports it. Every function works on a synth.State in place (its arrays are
the FP64 fields the reference's Array members hold).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from atsat_gb300 import abi, fields as F

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "atsat_oracle.c")
# The parity oracle: -O2 and no multiply-add contraction, so that on x86-64 it equals the reference bit for
# bit. ATSAT_ORACLE_BUILD=fast selects a second build used only as a timed CPU baseline: -O3 with
# contraction allowed (fused multiply-adds wherever the host ISA has them; no -march / -mcpu).
FAST = os.environ.get("ATSAT_ORACLE_BUILD", "") == "fast"
LIB_O2 = os.path.join(HERE, "liboracle.so")
LIB_FAST = os.path.join(HERE, "liboracle_fast.so")
CFLAGS_O2 = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c99", "-Wall"]
CFLAGS_FAST = ["-O3", "-fopenmp", "-ffp-contract=fast", "-fPIC", "-shared", "-std=c99", "-Wall"]
LIB = LIB_FAST if FAST else LIB_O2


def build(force: bool = False, fast: bool = FAST) -> str:
    lib, flags = (LIB_FAST, CFLAGS_FAST) if fast else (LIB_O2, CFLAGS_O2)
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < os.path.getmtime(SRC):
        subprocess.run(["gcc", *flags, SRC, "-o", lib, "-lm"], check=True)
    return lib


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
    return _lib


class _Call:
    def __init__(self, state, params: dict):
        self.state = state
        g = state.grid
        self.gh = abi.GridHold(g)
        self.p = abi.make_params(params)
        shape = g.shape
        for fid in range(F.NFIELDS):
            if fid not in state.arrays:
                state.arrays[fid] = np.zeros(shape)
        self.ptrs = (C.POINTER(C.c_double) * F.NFIELDS)()
        for fid in range(F.NFIELDS):
            a = state.arrays[fid]
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == shape
            self.ptrs[fid] = abi.dptr(a)
        self.buoy = np.zeros(g.im)

    def tables(self):
        s = self.state
        return (abi.dptr(s.cell_vbar0), abi.dptr(s.cell_ubar0), abi.dptr(s.p_baro))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def rhs(state, params) -> np.ndarray:
    c = _Call(state, params)
    _check(lib().orc_rhs(C.byref(c.gh.s), C.byref(c.p), c.ptrs, *c.tables(), abi.dptr(c.buoy)), "rhs")
    return c.buoy


def rk4_step(state, params) -> np.ndarray:
    c = _Call(state, params)
    _check(lib().orc_rk4_step(C.byref(c.gh.s), C.byref(c.p), c.ptrs, *c.tables(), abi.dptr(c.buoy)), "rk4")
    return c.buoy


def pressure(state, params) -> abi.PStats:
    c = _Call(state, params)
    st = abi.PStats()
    _check(lib().orc_pressure(C.byref(c.gh.s), C.byref(c.p), c.ptrs, C.byref(st)), "pressure")
    return st


def mixture_density(state, params):
    c = _Call(state, params)
    _check(lib().orc_mixture_density(C.byref(c.gh.s), C.byref(c.p), c.ptrs), "density")


def restore_var(state, params):
    c = _Call(state, params)
    _check(lib().orc_restore_var(C.byref(c.gh.s), C.byref(c.p), c.ptrs), "restore_var")


def buoyancy_ref_level(state, params) -> np.ndarray:
    c = _Call(state, params)
    _check(lib().orc_buoyancy_ref_level(C.byref(c.gh.s), C.byref(c.p), c.ptrs, abi.dptr(c.buoy)), "buoy")
    return c.buoy


def metric_pressure(state, params):
    c = _Call(state, params)
    _check(lib().orc_metric_pressure(C.byref(c.gh.s), C.byref(c.p), c.ptrs, abi.dptr(state.p_baro)), "metric")


def boundary_conditions(state, params):
    """bcTheta, bcPhi, bcRadius of BC_Sat on the dycore fields (cSaturnModel.cpp:1091-1093)."""
    c = _Call(state, params)
    _check(lib().orc_boundary_conditions(C.byref(c.gh.s), C.byref(c.p), c.ptrs), "bc")


def damp_wiggles(state, params, fid: int, along_i: bool, along_j: bool, along_k: bool, strength: float = 1.0,
                 passes: int = 1):
    """AtomUtils::damp_wiggles (lib/Utils.cpp:229-322) on one field, no surface mask."""
    c = _Call(state, params)
    _check(lib().orc_damp_wiggles(C.byref(c.gh.s), C.byref(c.p), c.ptrs, int(fid), int(along_i), int(along_j),
                                  int(along_k), C.c_double(strength), int(passes)), "damp_wiggles")


def damp_pdyn(state, params):
    """The p_dyn filter of cSaturnModel::Run after the pressure call (cSaturnModel.cpp:894-897)."""
    c = _Call(state, params)
    _check(lib().orc_damp_pdyn(C.byref(c.gh.s), C.byref(c.p), c.ptrs), "damp_pdyn")


def clamp_negative_species(state, params, budget=None):
    """cSaturnModel::clampNegativeSpecies (FileIO_Sat.cpp:716-772). budget: a float64 array of 44 (the
    clipped amount, the cells, and both for the radial planes, 11 species each) that is added to."""
    c = _Call(state, params)
    b = budget if budget is not None else np.zeros(44)
    _check(lib().orc_clamp_negative_species(C.byref(c.gh.s), C.byref(c.p), c.ptrs, abi.dptr(b)), "clamp")
    return b


def turbulence(state, params, tparams=None):
    """Turbulence<cSaturnModel>::run (Turbulence.h:306-329). Returns (prod, vel_star)."""
    c = _Call(state, params)
    tp = tparams if tparams is not None else abi.make_turb_params()
    g = state.grid
    prod = np.zeros(g.shape)
    vs = np.zeros((g.jm, g.km))
    _check(lib().orc_turbulence(C.byref(c.gh.s), C.byref(c.p), c.ptrs, C.byref(tp), abi.dptr(prod), abi.dptr(vs)),
           "turbulence")
    return prod, vs


def steps(state, params, nsteps: int, iter0: int = 1, glue: bool = False, budget=None, tparams=None):
    """The dycore sequence of cSaturnModel::Run (cSaturnModel.cpp:864-1111 restricted to the dycore):
    density + pressure on even iterations, RK4, boundary conditions, restoreVar. glue: also the driver's
    p_dyn filter after the pressure call, the species floor after the boundary conditions and the
    turbulence closure after restoreVar (cSaturnModel.cpp:894-897, 1101, 1116)."""
    for it in range(iter0, iter0 + nsteps):
        if it % 2 == 0:
            mixture_density(state, params)
            pressure(state, params)
            if glue:
                damp_pdyn(state, params)
        rk4_step(state, params)
        boundary_conditions(state, params)
        if glue:
            clamp_negative_species(state, params, budget)
        restore_var(state, params)
        if glue and params.get("turb_active", 1):
            turbulence(state, params, tparams)
