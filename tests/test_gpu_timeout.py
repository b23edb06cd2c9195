"""The timeout path of the TMA-tiled stage kernels' bounded waits (the status convention's
ATSAT_DYN_E_TIMEOUT), exercised without a GPU fault.

The test lowers the waits' limit to 2^20 SM clocks (about half a millisecond) and has every block's
producer leave the last item of its stream unissued: a barrier that nothing completes. The consumers'
waits for that item run out, the blocks set the device status word and return (each producer first
waits for its own copies in flight, which always land), and the next synchronisation reports
ATSAT_DYN_E_TIMEOUT. The handle stays usable: with the hook cleared and the state uploaded again, the
next iterations follow the oracle.
"""
import pytest

from atsat_gb300 import abi, fields as F
from oracle import oracle

from helpers import case

pytestmark = pytest.mark.gpu

ALL = list(range(F.NFIELDS))


def test_bounded_wait_runs_out_and_the_handle_recovers():
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=3)
    ref = st.copy()
    oracle.steps(ref, P, 2)
    with dyn.Dycore(g, dict(P, precision=1)) as d:
        assert d.stage_variant() == dyn.Dycore.STAGE_MARCH
        d.load_state(st.copy())
        assert d.timeouts() == 0
        d.set_wait_test(clocks=1 << 20, withhold=1)
        with pytest.raises(dyn.DycoreError) as ei:
            d.iterate(1, 1)
        assert ei.value.status == abi.E_TIMEOUT, ei.value
        assert d.timeouts() == 1
        # the status word was cleared when it was read: a plain sync reports nothing more
        d.set_wait_test(0, 0)
        d.sync()
        assert d.timeouts() == 1
        s = st.copy()
        d.load_state(s)
        d.iterate(1, 2)
        d.download(ALL)
        assert d.timeouts() == 1
    for f in [F.U, F.V, F.W, F.T, F.P_DYN]:
        a, b = s.arrays[f], ref.arrays[f]
        e = float(abs(a - b).max() / abs(b).max())
        assert e <= 1e-6, (F.NAMES[f], e)


def test_wait_test_arguments_are_checked():
    from atsat_gb300 import dyn
    g, P, _ = case((9, 13, 17), seed=3)
    with dyn.Dycore(g, dict(P, precision=1)) as d:
        for clocks, withhold in [(-1, 0), ((1 << 31) + 1, 0), (0, -1), (0, 9)]:
            with pytest.raises(dyn.DycoreError) as ei:
                d.set_wait_test(clocks, withhold)
            assert ei.value.status == abi.E_INVALID
