"""The no-allocation buoyancy level mean (atsat_dyn_buoyancy_ref_level_noalloc).

The entry point serves callers that cannot call cudaMalloc themselves: a program whose pool allocator
owns all device memory, or a step loop that must not allocate on its critical path. These tests play
such a caller: the device inputs are buffers that already exist (a handle's field copies, or the
caller's own pitched buffers), the output goes into another existing device buffer, and the call itself
allocates nothing. The result must agree with the handle's atsat_dyn_buoyancy_ref_level and with the
oracle's computeBuoyancyRefLevel within the FP64 parity bar, on two calls in a row; a call on a smaller
grid after a larger one must not see the earlier call's scratch.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from atsat_gb300 import abi, fields as F
from oracle import oracle

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


def _rel(got, ref):
    return float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))


def _check_grid(shape, seed, calls=2):
    from atsat_gb300 import dyn
    L, fn = _entry()
    g, P, st = case(shape, seed=seed)
    want = oracle.buoyancy_ref_level(st.copy(), P)
    with dyn.Dycore(g, P) as d:
        d.load_state(st)
        d.computeBuoyancyRefLevel()
        ref = d.buoy_ref_level()
        assert _rel(ref, want) <= TOL_FP64
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
            assert _rel(got, ref) <= TOL_FP64, ("vs the handle", call, _rel(got, ref))
            assert _rel(got, want) <= TOL_FP64, ("vs the oracle", call, _rel(got, want))
        # beyond the fixed scratch: refused with its own status, before any device work
        rc = fn(t_ptr, ps_ptr, pitch, 513, g.jm, g.km, abi.dptr(the_z), P["g"], P["r_mix"], P["R_mix"],
                P["t_ref"], out_ptr, None)
        assert rc == abi.E_TOO_LARGE
        # a host array where device memory is expected: refused before any device work
        rc = fn(abi.dptr(st.arrays[F.T]), ps_ptr, pitch, g.im, g.jm, g.km, abi.dptr(the_z), P["g"], P["r_mix"],
                P["R_mix"], P["t_ref"], out_ptr, None)
        assert rc == abi.E_INVALID


def test_noalloc_level_mean_matches_the_handle_entry_point():
    _check_grid((41, 181, 361), seed=31)


def test_noalloc_smaller_grid_after_larger():
    _check_grid((21, 91, 181), seed=37)


def test_noalloc_callers_own_pitched_buffers():
    """A 5 x 7 x 9 grid in the caller's own device buffers with a row pitch of 16 > km: fewer latitude rows
    than the scratch has chunks (some chunks are empty), a level whose temperatures are all <= 0 or NaN
    (its mean is 0, as in the reference), twice in a row against the oracle."""
    torch = pytest.importorskip("torch")
    _, fn = _entry()
    g, P, st = case((5, 7, 9), seed=39)
    st.arrays[F.T][2] = -1.0
    st.arrays[F.T][2, 1, 3] = np.nan
    st.arrays[F.T][3, 4, 5] = np.nan
    want = oracle.buoyancy_ref_level(st.copy(), P)
    assert want[2] == 0.0 and np.all(want[[0, 1, 3, 4]] != 0.0)
    pitch = 16
    dev = torch.device("cuda:0")

    def pitched(a):
        buf = torch.full((g.im, g.jm, pitch), np.nan, dtype=torch.float64)
        buf[:, :, : g.km] = torch.from_numpy(a)
        return buf.to(dev)

    t_d, ps_d = pitched(st.arrays[F.T]), pitched(st.arrays[F.P_STAT])
    out_d = torch.full((g.im,), np.nan, dtype=torch.float64, device=dev)
    the_z = np.ascontiguousarray(g.the_z, dtype=np.float64)
    torch.cuda.synchronize()
    for call in range(2):
        rc = fn(t_d.data_ptr(), ps_d.data_ptr(), pitch, g.im, g.jm, g.km, abi.dptr(the_z), P["g"], P["r_mix"],
                P["R_mix"], P["t_ref"], out_d.data_ptr(), None)
        assert rc == abi.OK, rc
        got = out_d.cpu().numpy()
        assert got[2] == 0.0, got
        assert _rel(got, want) <= TOL_FP64, (call, got, want)
        out_d.fill_(np.nan)
        torch.cuda.synchronize()
