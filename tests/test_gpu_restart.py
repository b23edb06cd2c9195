"""Restart files from and into device buffers (cSaturnModel::save_state / load_state,
planet/FileIO_Sat.cpp:513-695): the device's writer against the format's restatement (oracle/sat3.py,
which equals the reference's own files byte for byte, tests/test_oracle_golden.py), its reader on all
three formats, and the finiteness check."""
import os

import numpy as np
import pytest

from atsat_gb300 import fields as F
from oracle import sat3

from helpers import case

pytestmark = pytest.mark.gpu
ALL = list(range(F.NFIELDS))


def host_arrays(shape, seed):
    rng = np.random.default_rng(seed)
    return [rng.normal(size=shape) for _ in range(15)]


@pytest.mark.parametrize("shape", [(9, 13, 17), (12, 40, 70)])
@pytest.mark.parametrize("fmt", [3, 1])
@pytest.mark.parametrize("with_host", [True, False])
def test_device_writer_bytes(tmp_path, shape, fmt, with_host):
    from atsat_gb300 import dyn
    g, P, st = case(shape, seed=51)
    host = host_arrays(shape, 52) if with_host else None
    ref = str(tmp_path / "ref.bin")
    sat3.write(ref, st.arrays, host, g.shape, 77, fmt)
    out = str(tmp_path / "dev.bin")
    with dyn.Dycore(g, P) as d:
        d.load_state(st.copy())
        d.save_restart(out, 77, carried=(fmt == 3), host=host)
    assert open(out, "rb").read() == open(ref, "rb").read()


@pytest.mark.parametrize("fmt", [3, 2, 1])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_device_reader(tmp_path, fmt, precision):
    from atsat_gb300 import dyn
    g, P, st = case((12, 40, 70), seed=53)
    _, _, src = case((12, 40, 70), seed=54)          # what the file holds
    host = host_arrays(g.shape, 55)
    path = str(tmp_path / "r.bin")
    sat3.write(path, src.arrays, host, g.shape, 4321, fmt)
    got_host = [np.zeros(g.shape) for _ in range(15)]
    s = st.copy()
    with dyn.Dycore(g, dict(P, precision=precision)) as d:
        d.load_state(s)
        d.iterate(1, 2)                               # a resident state (aliased in the mixed path)
        it, f = d.load_restart(path, host=got_host)
        d.download(ALL)
    assert (it, f) == (4321, fmt)
    listed = [e for e in sat3.order(fmt) if not isinstance(e, tuple)]
    for fid in listed:
        assert np.array_equal(s.arrays[fid], src.arrays[fid]), F.NAMES[fid]
    for n in range(15):
        carried_host = fmt >= 2
        assert np.array_equal(got_host[n], host[n] if carried_host else np.zeros(g.shape))


def test_round_trip_then_iterate(tmp_path):
    """Resume = straight run: iterations 1-2, save, a fresh handle loads and runs 3-4, against 1-4 in one go."""
    from atsat_gb300 import dyn
    g, P, st = case((10, 20, 36), seed=57)
    path = str(tmp_path / "mid.bin")
    a = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(a)
        d.iterate(1, 2)
        d.save_restart(path, 2)
        d.iterate(3, 2)
        d.download(ALL)
    b = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(b)
        assert d.load_restart(path) == (2, 3)
        d.iterate(3, 2)
        d.download(ALL)
    for fid in F.PROG + [F.P_DYN, F.P_DYNN]:
        assert np.array_equal(a.arrays[fid], b.arrays[fid]), F.NAMES[fid]


def test_reader_rejects(tmp_path):
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=59)
    good = str(tmp_path / "good.bin")
    sat3.write(good, st.arrays, None, g.shape, 1, 3)
    other = str(tmp_path / "other.bin")
    g2, _, st2 = case((9, 13, 19), seed=59)
    sat3.write(other, st2.arrays, None, g2.shape, 1, 3)
    short = str(tmp_path / "short.bin")
    open(short, "wb").write(open(good, "rb").read()[:-8])
    bad = str(tmp_path / "bad.bin")
    raw = bytearray(open(good, "rb").read())
    raw[0:4] = np.array([0x53415439], dtype=np.int32).tobytes()
    open(bad, "wb").write(bytes(raw))
    with dyn.Dycore(g, P) as d:
        d.load_state(st.copy())
        for p in (other, short, bad, str(tmp_path / "missing.bin")):
            with pytest.raises(dyn.DycoreError):
                d.load_restart(p)
        assert d.load_restart(good) == (1, 3)


def test_restart_state_is_clean():
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=61)
    with dyn.Dycore(g, P) as d:
        d.load_state(st.copy())
        assert d.restart_state_is_clean()
    s = st.copy()
    s.arrays[F.RHS_T][2, 3, 4] = np.inf                 # not a restart array
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        assert d.restart_state_is_clean()
    s.arrays[F.ID["disn"]][1, 2, 3] = np.nan
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        assert not d.restart_state_is_clean()
