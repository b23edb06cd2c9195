"""Host bindings moved by the SMs in place (NVLink-C2C, the CPU's page tables) against the copy engines.

Upload and download are pure data movement, so both paths must give back exactly the bytes the host
holds: bitwise round trips for contiguous arrays, for the reference's ragged rows (one allocation of km
doubles per (i, j), lib/Array.cpp:62-70) and for rows that are views into one block, at a padded and an
unpadded grid, plus a dycore step fed through each path.
"""
import numpy as np
import pytest

from atsat_gb300 import fields as F

from helpers import TOL_FP64, case, compare

pytestmark = pytest.mark.gpu

FIELDS = [F.U, F.T, F.P_DYN, F.H2O, F.NUE]


def need_direct(d):
    if not d.host_direct():
        pytest.skip("the device does not address host memory in place here")


def rand_field(g, seed):
    return np.random.default_rng(seed).standard_normal(g.shape)


@pytest.mark.parametrize("shape", [(9, 13, 17), (21, 91, 181), (9, 13, 64)])   # kp > km twice, kp == km once
@pytest.mark.parametrize("direct_up,direct_down", [(True, True), (True, False), (False, True), (False, False)])
def test_array_round_trip(shape, direct_up, direct_down):
    from atsat_gb300 import dyn
    g, P, _ = case(shape, seed=3)
    with dyn.Dycore(g, P) as d:
        if direct_up or direct_down:
            need_direct(d)
        src = {fid: rand_field(g, 10 + fid) for fid in FIELDS}
        d.set_host_direct(direct_up)
        for fid in FIELDS:
            d.bind(fid, src[fid])
            assert d.host_direct(fid) == direct_up
        d.upload(FIELDS)
        out = {fid: np.full(g.shape, -7.0) for fid in FIELDS}
        d.set_host_direct(direct_down)
        for fid in FIELDS:
            d.bind(fid, out[fid])
        d.download(FIELDS)
    for fid in FIELDS:
        assert np.array_equal(out[fid], src[fid]), fid


@pytest.mark.parametrize("shape", [(9, 13, 17), (21, 91, 181)])
@pytest.mark.parametrize("direct", [True, False])
def test_ragged_rows_round_trip(shape, direct):
    """Separately allocated rows with a guard value past km that no transfer may touch."""
    from atsat_gb300 import dyn
    g, P, _ = case(shape, seed=4)
    n = g.im * g.jm
    with dyn.Dycore(g, P) as d:
        if direct:
            need_direct(d)
        d.set_host_direct(direct)
        src = {fid: rand_field(g, 20 + fid) for fid in FIELDS}
        rows_in, rows_out = {}, {}
        for fid in FIELDS:
            rows_in[fid] = [np.array(src[fid][r // g.jm, r % g.jm], copy=True) for r in range(n)]
            d.bind_rows(fid, rows_in[fid])
            assert d.host_direct(fid) == direct
        d.upload(FIELDS)
        for fid in FIELDS:
            bufs = [np.full(g.km + 3, 5.0) for _ in range(n)]
            rows_out[fid] = bufs
            d.bind_rows(fid, [b[:g.km] for b in bufs])
        d.download(FIELDS)
    for fid in FIELDS:
        got = np.stack([b[:g.km] for b in rows_out[fid]]).reshape(g.shape)
        assert np.array_equal(got, src[fid]), fid
        assert all(np.all(b[g.km:] == 5.0) for b in rows_out[fid]), fid


def test_rows_as_views_and_mixed_bindings():
    """Rows that are views into one block, next to contiguous arrays, in one upload and one download."""
    from atsat_gb300 import dyn
    g, P, _ = case((9, 13, 17), seed=5)
    with dyn.Dycore(g, P) as d:
        need_direct(d)
        a = rand_field(g, 31)
        b = rand_field(g, 32)
        d.bind_rows(F.U, [a[i, j] for i in range(g.im) for j in range(g.jm)])
        d.bind(F.V, b)
        d.upload([F.U, F.V])
        a2, b2 = np.zeros(g.shape), np.zeros(g.shape)
        d.bind(F.U, a2)
        d.bind_rows(F.V, [b2[i, j] for i in range(g.im) for j in range(g.jm)])
        d.download([F.U, F.V])
    assert np.array_equal(a2, a) and np.array_equal(b2, b)


@pytest.mark.parametrize("direct", [True, False])
def test_rk_step_through_each_path(direct):
    """One RK4 step fed and read back through one path; both agree with the oracle at the FP64 bar."""
    from atsat_gb300 import dyn
    from oracle import oracle
    g, P, st = case((9, 13, 17), seed=17)
    ref = st.copy()
    oracle.rk4_step(ref, P)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        if direct:
            need_direct(d)
        d.set_host_direct(direct)
        rows = {}
        for fid in range(F.NFIELDS):
            a = s.arrays[fid]
            rows[fid] = [np.array(a[i, j], copy=True) for i in range(g.im) for j in range(g.jm)]
            d.bind_rows(fid, rows[fid])
        d.upload(list(range(F.NFIELDS)))
        d.set_tables(s.cell_vbar0, s.cell_ubar0)
        d.RungeKuttaSat()
        d.download(list(range(F.NFIELDS)))
    got = {fid: np.stack(rows[fid]).reshape(g.shape) for fid in range(F.NFIELDS)}
    compare(got, ref.arrays, F.PROG + [F.RHS_U, F.RHS_V, F.RHS_W], TOL_FP64, "rk step")


def test_misaligned_rows_take_the_copy_engines():
    """A row pointer that is not a whole double (8-byte aligned) sends its binding to the copy engines; the
    round trip is still exact."""
    from atsat_gb300 import dyn
    g, P, _ = case((9, 13, 17), seed=6)
    n = g.im * g.jm
    src = rand_field(g, 41)
    with dyn.Dycore(g, P) as d:
        need_direct(d)
        raw = [np.zeros(g.km * 8 + 8, dtype=np.uint8) for _ in range(n)]
        rows = []
        for r in range(n):
            off = 4 if r == 7 else 0
            a = raw[r][off:off + g.km * 8].view(np.float64)
            a[...] = src[r // g.jm, r % g.jm]
            rows.append(a)
        d.bind_rows(F.T, rows)
        assert not d.host_direct(F.T)
        d.upload([F.T])
        out = np.zeros(g.shape)
        d.bind(F.T, out)
        assert d.host_direct(F.T)
        d.download([F.T])
    assert np.array_equal(out, src)


def test_async_step_equals_sync():
    """A host-fed step queued in the asynchronous mode (upload, density, pressure without statistics, RK4,
    download, then one sync) gives the synchronous mode's bits."""
    from atsat_gb300 import dyn
    g, P, st = case((21, 91, 181), seed=8)
    outs = F.PROG + [F.RHS_U, F.RHS_V, F.RHS_W, F.AUX_U, F.AUX_V, F.AUX_W, F.P_DYN]
    res = []
    for mode in (False, True):
        s = st.copy()
        with dyn.Dycore(g, dict(P, precision=1)) as d:
            d.load_state(s)
            d.set_async(mode)
            for it in (2, 3):
                d.upload(list(range(F.NFIELDS)))
                if it % 2 == 0:
                    d.computeMixtureDensity()
                    d.PressureSolver_run(stats=False)
                d.RungeKuttaSat()
                d.download(outs)
                d.sync()
        res.append(s)
    for fid in outs:
        assert np.array_equal(res[0].arrays[fid], res[1].arrays[fid], equal_nan=True), F.NAMES[fid]
