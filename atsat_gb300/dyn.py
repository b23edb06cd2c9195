"""Host-side mirror of the ATSAT dynamical-core interface over the C ABI (include/atsat_dyn.h).

`Dycore` stands for the part of cSaturnModel this library replaces. Its methods keep the reference's
names and meaning:

    RungeKuttaSat()                 cSaturnModel::RungeKuttaSat        RungeKutta_Sat_Turb.cpp:110-387
    PressureSolver_run()            PressureSolver<cSaturnModel>::run  PressureSolver.h:145-766
    computeMixtureDensity()         cSaturnModel::computeMixtureDensity Pressure_Sat.cpp:49-62
    computeBuoyancyRefLevel()       RungeKutta_Sat_Turb.cpp:31-50
    computeMetricPressure()         RungeKutta_Sat_Turb.cpp:60-108
    RHSSat_pass()                   one RHSSat pass over the RK interior (:220-247)
    prepareProjectionBoundaries()   Pressure_Sat.cpp:78-194
    restoreVar()                    cSaturnModel::restoreVar(1.0)      cSaturnModel.cpp:1551-1600
    boundary_conditions()           BC_Sat bcTheta, bcPhi, bcRadius    cSaturnModel.cpp:1091-1093

Fields live on the device; `bind`/`upload`/`download` move them to and from host numpy arrays (the
reference's Array storage). Every call raises DycoreError on a non-zero status: there is no CPU
fallback, and a missing CUDA build is an ImportError-like failure at load time.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi, fields as F

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libatsat_dyn.so")

_lib = None


class DycoreError(RuntimeError):
    def __init__(self, status: int, what: str, msg: str):
        super().__init__(f"{what}: status {status}: {msg}")
        self.status = status


def lib():
    """The loaded CUDA library. Raises if it has not been built: the product has no CPU path."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libatsat_dyn.so is not built ({LIB_PATH}); run "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        L.atsat_dyn_create.argtypes = [C.POINTER(abi.Grid), C.POINTER(abi.Params), C.POINTER(H)]
        L.atsat_dyn_destroy.argtypes = [H]
        L.atsat_dyn_destroy.restype = None
        L.atsat_dyn_last_error.argtypes = [H]
        L.atsat_dyn_last_error.restype = C.c_char_p
        L.atsat_dyn_params_default.argtypes = [C.POINTER(abi.Params)]
        L.atsat_dyn_params_from_env.argtypes = [C.POINTER(abi.Params)]
        L.atsat_dyn_bind_host_rows.argtypes = [H, C.c_int32, C.POINTER(C.POINTER(C.c_double))]
        L.atsat_dyn_bind_host_array.argtypes = [H, C.c_int32, C.POINTER(C.c_double)]
        L.atsat_dyn_upload.argtypes = [H, C.POINTER(C.c_int32), C.c_int32]
        L.atsat_dyn_download.argtypes = [H, C.POINTER(C.c_int32), C.c_int32]
        L.atsat_dyn_set_host_direct.argtypes = [H, C.c_int32]
        L.atsat_dyn_set_async.argtypes = [H, C.c_int32]
        L.atsat_dyn_host_direct.argtypes = [H, C.c_int32]
        L.atsat_dyn_set_tables.argtypes = [H, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.atsat_dyn_get_buoy_ref_level.argtypes = [H, C.POINTER(C.c_double)]
        for n in ("mixture_density", "buoyancy_ref_level", "metric_pressure", "rhs", "rk4_step",
                  "prepare_projection_boundaries", "restore_var", "sync", "boundary_conditions"):
            fn = getattr(L, "atsat_dyn_" + n, None)
            if fn is not None:
                fn.argtypes = [H]
        L.atsat_dyn_pressure.argtypes = [H, C.POINTER(abi.PStats)]
        L.atsat_dyn_iterate.argtypes = [H, C.c_int32, C.c_int32]
        L.atsat_dyn_status.argtypes = [H, C.POINTER(abi.Diag)]
        L.atsat_dyn_count_nonfinite.argtypes = [H, C.c_int32, C.POINTER(C.c_int64)]
        L.atsat_dyn_profile.argtypes = [H, C.c_int32]
        L.atsat_dyn_profile_classes.argtypes = [H, C.c_uint32]
        L.atsat_dyn_profile_reset.argtypes = [H]
        L.atsat_dyn_profile_read.argtypes = [H, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.atsat_dyn_device_field.argtypes = [H, C.c_int32, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int64)]
        L.atsat_dyn_host_alloc.argtypes = [C.c_size_t]
        L.atsat_dyn_host_alloc.restype = C.c_void_p
        L.atsat_dyn_host_free.argtypes = [C.c_void_p]
        L.atsat_dyn_host_free.restype = None
        L.atsat_dyn_set_write_all_rhs.argtypes = [H, C.c_int32]
        L.atsat_dyn_set_wait_test.argtypes = [H, C.c_int64, C.c_int32]
        L.atsat_dyn_set_stage_variant.argtypes = [H, C.c_int32]
        L.atsat_dyn_get_stage_variant.argtypes = [H, C.POINTER(C.c_int32)]
        L.atsat_dyn_set_march_levels.argtypes = [H, C.c_int32]
        L.atsat_dyn_get_march_levels.argtypes = [H, C.POINTER(C.c_int32)]
        L.atsat_dyn_tune_cache_get.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint32, C.c_char_p,
                                               C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.atsat_dyn_tune_cache_put.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_uint32, C.c_char_p,
                                               C.c_int32, C.c_int32, C.c_double]
        L.atsat_dyn_autotune.argtypes = [H, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.atsat_dyn_graph_capture.argtypes = [H, C.c_int32, C.c_int32]
        L.atsat_dyn_graph_launch.argtypes = [H, C.c_int32]
        L.atsat_dyn_ensemble_run.argtypes = [C.POINTER(H), C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_double)]
        L.atsat_dyn_poisson_project.argtypes = [H, C.POINTER(C.c_double)]
        L.atsat_dyn_poisson_solve.argtypes = [H, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double,
                                              C.c_int32, C.c_int32, C.c_double, C.POINTER(abi.PoissonStats)]
        L.atsat_dyn_timer_start.argtypes = [H]
        L.atsat_dyn_timer_stop.argtypes = [H, C.POINTER(C.c_double)]
        L.atsat_dyn_conv_selftest.argtypes = [C.c_int32, C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.atsat_dyn_damp_wiggles.argtypes = [H, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_int32]
        L.atsat_dyn_damp_pdyn.argtypes = [H]
        L.atsat_dyn_turb_params_default.argtypes = [C.POINTER(abi.TurbParams)]
        L.atsat_dyn_turb_params_from_env.argtypes = [C.POINTER(abi.TurbParams)]
        L.atsat_dyn_set_turb_params.argtypes = [H, C.POINTER(abi.TurbParams)]
        L.atsat_dyn_turbulence.argtypes = [H]
        L.atsat_dyn_save_restart.argtypes = [H, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(C.POINTER(C.c_double))]
        L.atsat_dyn_load_restart.argtypes = [H, C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                             C.POINTER(C.POINTER(C.c_double))]
        L.atsat_dyn_restart_is_clean.argtypes = [H, C.POINTER(C.c_int32)]
        L.atsat_dyn_turbulence_diag.argtypes = [H, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.atsat_dyn_clamp_negative_species.argtypes = [H]
        L.atsat_dyn_clamp_budget.argtypes = [H, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                             C.POINTER(C.c_int64)]
        _lib = L
    return _lib


def conv_selftest(n_doubles: int = 1 << 32, device: int = 0) -> tuple[int, int]:
    """Mismatches of the integer-pipe float<->double conversions against the hardware's (widening over
    all 2^32 floats, narrowing over those and n_doubles hashed doubles); (0, 0) means bit-identical."""
    w, n = C.c_uint64(0), C.c_uint64(0)
    rc = lib().atsat_dyn_conv_selftest(device, n_doubles, C.byref(w), C.byref(n))
    if rc != 0:
        raise DycoreError(rc, "atsat_dyn_conv_selftest", "CUDA error")
    return w.value, n.value


def params_from_env(base: dict | None = None) -> dict:
    """The reference's constants (`base`, default: its committed configuration) with every knob
    resolved from the ATSAT_* environment as the reference resolves it."""
    p = abi.make_params(base or abi.default_params())
    rc = lib().atsat_dyn_params_from_env(C.byref(p))
    if rc != 0:
        raise DycoreError(rc, "atsat_dyn_params_from_env", "an ATSAT_* knob is set to a value with no device path")
    out = {n: getattr(p, n) for n, _ in F.PARAM_DOUBLES}
    out.update({n: getattr(p, n) for n, _ in F.PARAM_INTS})
    return out


class PinnedArray:
    """A numpy array over page-locked host memory (cudaHostAlloc), for fast host<->device copies."""

    def __init__(self, shape, dtype=np.float64):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = lib().atsat_dyn_host_alloc(max(n, 8))
        if not self._p:
            raise MemoryError("cudaHostAlloc failed")
        buf = (C.c_char * n).from_address(self._p)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            lib().atsat_dyn_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Dycore:
    def __init__(self, grid, params: dict):
        self.grid = grid
        self._gh = abi.GridHold(grid)
        self._p = abi.make_params(params)
        self.params = dict(params)
        self.h = C.c_void_p()
        self._bound = {}
        rc = lib().atsat_dyn_create(C.byref(self._gh.s), C.byref(self._p), C.byref(self.h))
        if rc != 0:
            msg = lib().atsat_dyn_last_error(self.h).decode() if self.h else ""
            self.close()
            raise DycoreError(rc, "atsat_dyn_create", msg)

    # ---- plumbing ----
    def _ck(self, rc, what):
        if rc != 0:
            raise DycoreError(rc, what, lib().atsat_dyn_last_error(self.h).decode())

    def close(self):
        if self.h:
            lib().atsat_dyn_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def bind(self, fid: int, arr: np.ndarray):
        assert arr.dtype == np.float64 and arr.flags.c_contiguous and arr.shape == self.grid.shape
        self._bound[fid] = arr
        self._ck(lib().atsat_dyn_bind_host_array(self.h, fid, abi.dptr(arr)), "bind_host_array")

    def bind_rows(self, fid: int, rows: list):
        """Bind the reference's ragged storage: rows[i*jm + j] is a float64 array of km values."""
        n = self.grid.im * self.grid.jm
        assert len(rows) == n
        ptrs = (C.POINTER(C.c_double) * n)(*[abi.dptr(r) for r in rows])
        self._bound[fid] = (rows, ptrs)
        self._ck(lib().atsat_dyn_bind_host_rows(self.h, fid, ptrs), "bind_host_rows")

    def bind_state(self, state, fids=None):
        for fid in (fids if fids is not None else range(F.NFIELDS)):
            if fid not in state.arrays:
                state.arrays[fid] = np.zeros(self.grid.shape)
            self.bind(fid, state.arrays[fid])

    def upload(self, fids):
        ids = (C.c_int32 * len(fids))(*fids)
        self._ck(lib().atsat_dyn_upload(self.h, ids, len(fids)), "upload")

    def download(self, fids):
        ids = (C.c_int32 * len(fids))(*fids)
        self._ck(lib().atsat_dyn_download(self.h, ids, len(fids)), "download")

    def set_host_direct(self, enable: bool):
        """Move bound fields with one kernel that reads / writes host memory in place (NVLink-C2C, the
        CPU's page tables), or with the copy engines through staging buffers."""
        self._ck(lib().atsat_dyn_set_host_direct(self.h, 1 if enable else 0), "set_host_direct")

    def host_direct(self, fid: int = -1) -> bool:
        """Whether field fid's binding (fid -1: the handle) takes the in-place path."""
        r = lib().atsat_dyn_host_direct(self.h, fid)
        self._ck(min(r, 0), "host_direct")
        return r == 1

    def set_tables(self, cell_vbar0=None, cell_ubar0=None, p_baro=None):
        self._tables = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                        for a in (cell_vbar0, cell_ubar0, p_baro)]
        self._ck(lib().atsat_dyn_set_tables(self.h, *[abi.dptr(a) for a in self._tables]), "set_tables")

    def load_state(self, state):
        """Bind every field of a synth.State, upload it and set its tables."""
        self.bind_state(state)
        self.upload(list(range(F.NFIELDS)))
        self.set_tables(state.cell_vbar0, state.cell_ubar0, state.p_baro)

    def buoy_ref_level(self) -> np.ndarray:
        out = np.zeros(self.grid.im)
        self._ck(lib().atsat_dyn_get_buoy_ref_level(self.h, abi.dptr(out)), "get_buoy_ref_level")
        return out

    def set_write_all_rhs(self, on: bool):
        self._ck(lib().atsat_dyn_set_write_all_rhs(self.h, int(bool(on))), "set_write_all_rhs")

    (STAGE_DIRECT, STAGE_TILED, STAGE_SPLIT, STAGE_SPLIT3, STAGE_SPLIT13, STAGE_SPLIT_TILED, STAGE_TILED2,
     STAGE_MARCH) = range(8)
    STAGE_NAMES = ["direct", "tiled", "split", "split3", "split13", "split_tiled", "tiled2", "march"]

    def set_stage_variant(self, variant: int):
        """Mixed precision: the RK stage kernel (STAGE_* constants)."""
        self._ck(lib().atsat_dyn_set_stage_variant(self.h, int(variant)), "set_stage_variant")

    def stage_variant(self) -> int:
        v = C.c_int32(-1)
        self._ck(lib().atsat_dyn_get_stage_variant(self.h, C.byref(v)), "get_stage_variant")
        return v.value

    def set_march_levels(self, levels: int):
        """MARCH variant: radial levels per block (the march depth)."""
        self._ck(lib().atsat_dyn_set_march_levels(self.h, int(levels)), "set_march_levels")

    def march_levels(self) -> int:
        v = C.c_int32(0)
        self._ck(lib().atsat_dyn_get_march_levels(self.h, C.byref(v)), "get_march_levels")
        return v.value

    def tuned_from_cache(self) -> bool:
        d = abi.Diag()
        self._ck(lib().atsat_dyn_status(self.h, C.byref(d)), "status")
        return bool(d.tuned_from_cache)

    def autotune(self, reps: int = 10):
        """Time every available stage variant (the MARCH variant at several march depths) on this grid, keep
        the fastest and record it in the autotune cache; returns (chosen, ms per variant, -1 where
        unavailable)."""
        chosen = C.c_int32(-1)
        ms = (C.c_double * len(self.STAGE_NAMES))()
        self._ck(lib().atsat_dyn_autotune(self.h, int(reps), C.byref(chosen), ms), "autotune")
        return chosen.value, list(ms)

    # ---- CUDA graphs of the resident loop (no reference counterpart) ----
    def graph_capture(self, iter0: int, n: int = 2):
        """Record n resident iterations from iter0 into a CUDA graph (needs two resident iterations first)."""
        self._ck(lib().atsat_dyn_graph_capture(self.h, int(iter0), int(n)), "graph_capture")

    def graph_launch(self, reps: int = 1):
        """Enqueue `reps` replays of the captured graph (asynchronous; sync() waits)."""
        self._ck(lib().atsat_dyn_graph_launch(self.h, int(reps)), "graph_launch")

    # ---- standalone pressure-equation solves (no reference counterpart) ----
    def poisson_project(self, src: np.ndarray) -> np.ndarray:
        """A copy of `src` (im x jm x km) without its component outside the operator's range."""
        out = np.ascontiguousarray(src, dtype=np.float64).copy()
        assert out.shape == self.grid.shape
        self._ck(lib().atsat_dyn_poisson_project(self.h, abi.dptr(out)), "poisson_project")
        return out

    def poisson_solve(self, method, src: np.ndarray, tol: float = 1e-10, max_iter: int = 100, inner: int = 0,
                      omega: float = 1.0):
        """Solve L p = src with `method` (a name of abi.POISSON_METHODS or its index); returns (p, stats)."""
        m = abi.POISSON_METHODS.index(method) if isinstance(method, str) else int(method)
        f = np.ascontiguousarray(src, dtype=np.float64)
        assert f.shape == self.grid.shape
        p = np.zeros(self.grid.shape)
        st = abi.PoissonStats()
        self._ck(lib().atsat_dyn_poisson_solve(self.h, m, abi.dptr(f), abi.dptr(p), float(tol), int(max_iter),
                                               int(inner), float(omega), C.byref(st)), "poisson_solve")
        return p, {"method": abi.POISSON_METHODS[m], "iterations": st.iterations, "inner": st.inner,
                   "converged": bool(st.converged), "rel_residual": st.rel_residual, "ms": st.ms,
                   "sweeps_per_pass": st.sweeps_per_pass, "sweep_ms": st.sweep_ms}

    # ---- the reference's entry points ----
    def computeMixtureDensity(self):
        self._ck(lib().atsat_dyn_mixture_density(self.h), "mixture_density")

    def computeBuoyancyRefLevel(self):
        self._ck(lib().atsat_dyn_buoyancy_ref_level(self.h), "buoyancy_ref_level")

    def computeMetricPressure(self):
        self._ck(lib().atsat_dyn_metric_pressure(self.h), "metric_pressure")

    def RHSSat_pass(self):
        self._ck(lib().atsat_dyn_rhs(self.h), "rhs")

    def RungeKuttaSat(self):
        self._ck(lib().atsat_dyn_rk4_step(self.h), "rk4_step")

    def prepareProjectionBoundaries(self):
        self._ck(lib().atsat_dyn_prepare_projection_boundaries(self.h), "prepare_projection_boundaries")

    def PressureSolver_run(self, stats: bool = True):
        """PressureSolver<cSaturnModel>::run; its statistics when `stats` (which waits for the call)."""
        st = abi.PStats() if stats else None
        self._ck(lib().atsat_dyn_pressure(self.h, C.byref(st) if stats else None), "pressure")
        return st

    def set_async(self, enable: bool):
        """Transfers and compute calls return once queued (sync() before touching bound arrays)."""
        self._ck(lib().atsat_dyn_set_async(self.h, 1 if enable else 0), "set_async")

    def damp_wiggles(self, fid: int, along_i: bool, along_j: bool, along_k: bool, strength: float = 1.0,
                     passes: int = 1):
        """AtomUtils::damp_wiggles on a device field (lib/Utils.cpp:229-322), no surface mask."""
        self._ck(lib().atsat_dyn_damp_wiggles(self.h, int(fid), int(along_i), int(along_j), int(along_k),
                                              float(strength), int(passes)), "damp_wiggles")

    def damp_pdyn(self):
        """The p_dyn filter of cSaturnModel::Run after the pressure call (cSaturnModel.cpp:894-897)."""
        self._ck(lib().atsat_dyn_damp_pdyn(self.h), "damp_pdyn")

    def set_turb_params(self, tp):
        """The closure's knobs (abi.TurbParams, e.g. abi.make_turb_params(model=1))."""
        self._ck(lib().atsat_dyn_set_turb_params(self.h, C.byref(tp)), "set_turb_params")

    def TurbulenceSat_run(self):
        """Turbulence<cSaturnModel>::run on the device fields (Turbulence.h:306-329)."""
        self._ck(lib().atsat_dyn_turbulence(self.h), "turbulence")

    def turbulence_diag(self):
        """(P_k over the grid, u_tau per (j, k)) after the last closure run."""
        g = self.grid
        prod = np.zeros(g.shape)
        vs = np.zeros((g.jm, g.km))
        self._ck(lib().atsat_dyn_turbulence_diag(self.h, abi.dptr(prod), abi.dptr(vs)), "turbulence_diag")
        return prod, vs

    def save_restart(self, path: str, iteration: int, carried: bool = True, host=None):
        """cSaturnModel::save_state's file (SAT3, or SAT1 without the carried arrays) from the device fields;
        host: the 15 host-physics arrays (ATSAT_DYN_RESTART_NHOST order) or None for zeros."""
        ptrs = self._host_ptrs(host)
        self._ck(lib().atsat_dyn_save_restart(self.h, path.encode(), int(iteration), int(bool(carried)), ptrs),
                 "save_restart")

    def load_restart(self, path: str, host=None):
        """cSaturnModel::load_state into the device fields (and the host arrays given); (iteration, format)."""
        it, fmt = C.c_int32(), C.c_int32()
        self._ck(lib().atsat_dyn_load_restart(self.h, path.encode(), C.byref(it), C.byref(fmt), self._host_ptrs(host)),
                 "load_restart")
        return it.value, fmt.value

    def restart_state_is_clean(self) -> bool:
        v = C.c_int32()
        self._ck(lib().atsat_dyn_restart_is_clean(self.h, C.byref(v)), "restart_is_clean")
        return bool(v.value)

    def _host_ptrs(self, host):
        if host is None:
            return None
        assert len(host) == 15
        for a in host:
            assert a is None or (a.dtype == np.float64 and a.flags.c_contiguous and a.shape == self.grid.shape)
        return (C.POINTER(C.c_double) * 15)(*[abi.dptr(a) if a is not None else None for a in host])

    def clampNegativeSpecies(self):
        self._ck(lib().atsat_dyn_clamp_negative_species(self.h), "clamp_negative_species")

    def clamp_budget(self) -> np.ndarray:
        """44 values: clipped amount, cells, clipped amount on the radial planes, cells there (11 species each)."""
        a, c = (C.c_double * 11)(), (C.c_int64 * 11)()
        ab, cb = (C.c_double * 11)(), (C.c_int64 * 11)()
        self._ck(lib().atsat_dyn_clamp_budget(self.h, a, c, ab, cb), "clamp_budget")
        return np.concatenate([np.array(a[:]), np.array(c[:], dtype=np.float64), np.array(ab[:]),
                               np.array(cb[:], dtype=np.float64)])

    def restoreVar(self):
        self._ck(lib().atsat_dyn_restore_var(self.h), "restore_var")

    def boundary_conditions(self):
        self._ck(lib().atsat_dyn_boundary_conditions(self.h), "boundary_conditions")

    def iterate(self, iter0: int, n: int):
        """n iterations of the dycore part of cSaturnModel::Run, resident on the device."""
        self._ck(lib().atsat_dyn_iterate(self.h, iter0, n), "iterate")

    # ---- diagnostics ----
    def sync(self):
        self._ck(lib().atsat_dyn_sync(self.h), "sync")

    def launches(self) -> int:
        d = abi.Diag()
        self._ck(lib().atsat_dyn_status(self.h, C.byref(d)), "status")
        return int(d.launches)

    def timeouts(self) -> int:
        """How many synchronisations found a bounded device wait that gave up."""
        d = abi.Diag()
        self._ck(lib().atsat_dyn_status(self.h, C.byref(d)), "status")
        return int(d.timeout)

    def set_wait_test(self, clocks: int = 0, withhold: int = 0):
        """Failure-detection test hook: the tiled kernels' waits give up after `clocks` SM clocks (0: the
        default 2^31), and each block's producer leaves its last `withhold` items unissued."""
        self._ck(lib().atsat_dyn_set_wait_test(self.h, int(clocks), int(withhold)), "set_wait_test")

    def count_nonfinite(self, fid: int) -> int:
        n = C.c_int64()
        self._ck(lib().atsat_dyn_count_nonfinite(self.h, fid, C.byref(n)), "count_nonfinite")
        return int(n.value)

    def timer_start(self):
        self._ck(lib().atsat_dyn_timer_start(self.h), "timer_start")

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._ck(lib().atsat_dyn_timer_stop(self.h, C.byref(ms)), "timer_stop")
        return float(ms.value)

    def profile(self, on: bool):
        self._ck(lib().atsat_dyn_profile(self.h, int(on)), "profile")

    def profile_classes(self, classes):
        """Profile only the given kernel classes (abi.K_* ids)."""
        mask = 0
        for c in classes:
            mask |= 1 << int(c)
        self._ck(lib().atsat_dyn_profile_classes(self.h, mask), "profile_classes")

    def profile_reset(self):
        self._ck(lib().atsat_dyn_profile_reset(self.h), "profile_reset")

    def profile_read(self, kclass: int):
        n, ms = C.c_int64(), C.c_double()
        self._ck(lib().atsat_dyn_profile_read(self.h, kclass, C.byref(n), C.byref(ms)), "profile_read")
        return int(n.value), float(ms.value)


def ensemble_run(members, reps: int, concurrent: bool = True) -> float:
    """Replay every member's captured graph `reps` times, concurrently (one stream per member) or one
    member after another; returns the device milliseconds of the whole set."""
    H = C.c_void_p
    arr = (H * len(members))(*[m.h for m in members])
    ms = C.c_double(0.0)
    rc = lib().atsat_dyn_ensemble_run(arr, len(members), int(reps), int(bool(concurrent)), C.byref(ms))
    if rc != 0:
        raise DycoreError(rc, "ensemble_run", lib().atsat_dyn_last_error(members[0].h).decode())
    return ms.value
