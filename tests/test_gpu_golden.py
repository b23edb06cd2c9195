"""The CUDA path at the reference's own grid (41x181x361) against the reference's fixtures."""
import numpy as np
import pytest

from atsat_gb300 import fields as F
from golden.make_golden import CASES, make_state

from golden_cases import check_inputs, check_outputs, load
from helpers import TOL_FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_against_reference_fixture(name):
    from atsat_gb300 import dyn
    op, nsteps, seed, exercise, over = CASES[name]
    g, P, st = make_state(name)
    rec = load(name)
    check_inputs(rec, st)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.set_write_all_rhs(True)
        if op == "rhs":
            d.computeBuoyancyRefLevel()
            d.computeMetricPressure()
            d.RHSSat_pass()
        elif op == "rk":
            d.RungeKuttaSat()
        elif op == "pressure":
            d.PressureSolver_run()
        elif op == "density":
            d.computeMixtureDensity()
        elif op == "steps":
            d.iterate(1, nsteps)
        d.download(list(range(F.NFIELDS)))
        buoy = d.buoy_ref_level()
    check_outputs(rec, s.arrays, TOL_FP64, name)
    if "buoy_ref_level" in rec:
        assert np.max(np.abs(buoy - rec["buoy_ref_level"])) <= TOL_FP64 * np.max(np.abs(rec["buoy_ref_level"]))
