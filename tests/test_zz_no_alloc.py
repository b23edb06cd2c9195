"""The no-allocation buoyancy level mean (atsat_dyn_buoyancy_ref_level_noalloc) against the handle's own.

The entry point serves callers that cannot call cudaMalloc themselves: a program whose pool allocator
owns all device memory, or a step loop that must not allocate on its critical path. This test plays
such a caller: its device inputs are device buffers that already exist (a handle's field copies), its
output goes into another existing device buffer, and the call itself allocates nothing. The result must
agree with atsat_dyn_buoyancy_ref_level within the FP64 parity bar, on two calls in a row, and a call
on a smaller grid after a larger one must not see the earlier call's scratch.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from atsat_gb300 import abi, fields as F

from helpers import TOL_FP64, case

pytestmark = pytest.mark.gpu


def _entry():
    from atsat_gb300 import dyn
    L = dyn.lib()
    f = L.atsat_dyn_buoyancy_ref_level_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_double),
                  C.c_double, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, f


def _device_field(L, h, fid):
    p = C.POINTER(C.c_double)()
    pitch = C.c_int64()
    assert L.atsat_dyn_device_field(h, fid, C.byref(p), C.byref(pitch)) == 0
    return C.cast(p, C.c_void_p).value, pitch.value


def _check_grid(shape, seed, calls=2):
    from atsat_gb300 import dyn
    L, fn = _entry()
    g, P, st = case(shape, seed=seed)
    with dyn.Dycore(g, P) as d:
        d.load_state(st)
        d.computeBuoyancyRefLevel()
        ref = d.buoy_ref_level()
        t_ptr, pitch = _device_field(L, d.h, F.T)
        ps_ptr, _ = _device_field(L, d.h, F.P_STAT)
        # the output: the first im doubles of the device copy of a field nothing here reads (Q_rad)
        out_ptr, _ = _device_field(L, d.h, F.Q_RAD)
        assert g.im <= g.km
        the_z = np.ascontiguousarray(g.the_z, dtype=np.float64)
        for call in range(calls):
            st.arrays[F.Q_RAD][...] = 0.0
            d.upload([F.Q_RAD])
            rc = fn(t_ptr, ps_ptr, pitch, g.im, g.jm, g.km, abi.dptr(the_z), P["g"], P["r_mix"], P["R_mix"],
                    P["t_ref"], out_ptr, None)
            assert rc == abi.OK, rc
            d.download([F.Q_RAD])
            got = st.arrays[F.Q_RAD][0, 0, : g.im].copy()
            err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
            assert err <= TOL_FP64, (call, err)
        # beyond the fixed scratch: refused with its own status, before any device work
        rc = fn(t_ptr, ps_ptr, pitch, 513, g.jm, g.km, abi.dptr(the_z), P["g"], P["r_mix"], P["R_mix"],
                P["t_ref"], out_ptr, None)
        assert rc == -8


def test_noalloc_level_mean_matches_the_handle_entry_point():
    _check_grid((41, 181, 361), seed=31)


def test_noalloc_smaller_grid_after_larger():
    _check_grid((21, 91, 181), seed=37)
