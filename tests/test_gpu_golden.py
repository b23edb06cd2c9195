"""The CUDA path at the reference's own grid (41x181x361) against the reference's fixtures."""
import numpy as np
import pytest

from atsat_gb300 import fields as F
from golden.make_golden import CASES, make_state

from golden_cases import check_closure_arrays, check_inputs, check_outputs, load
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
    budget = None
    with dyn.Dycore(g, dict(P, driver_glue=1) if op == "driver" else P) as d:
        d.load_state(s)
        d.set_write_all_rhs(True)
        if op in ("driver", "steps"):
            d.iterate(1, nsteps)
        elif op == "damp":
            d.damp_pdyn()
        elif op == "clamp":
            d.clampNegativeSpecies()
        elif op == "turb":
            from atsat_gb300 import abi
            from golden.make_golden import split_over
            d.set_turb_params(abi.make_turb_params(**split_over(over)[1]))
            d.TurbulenceSat_run()
            closure = d.turbulence_diag()
        elif op == "rhs":
            d.computeBuoyancyRefLevel()
            d.computeMetricPressure()
            d.RHSSat_pass()
        elif op == "rk":
            d.RungeKuttaSat()
        elif op == "pressure":
            d.PressureSolver_run()
        elif op == "density":
            d.computeMixtureDensity()
        d.download(list(range(F.NFIELDS)))
        buoy = d.buoy_ref_level()
        if op in ("clamp", "driver"):
            budget = d.clamp_budget()
    check_outputs(rec, s.arrays, TOL_FP64, name)
    if op == "turb":
        check_closure_arrays(rec, closure[0], closure[1], TOL_FP64)
    if budget is not None:
        rb = rec["clamp_budget"]
        n = len(rb) // 4
        # counts exactly (the cells a floor touches), amounts to the FP64 bar
        assert np.array_equal(budget[n:2 * n], rb[n:2 * n]) and np.array_equal(budget[3 * n:], rb[3 * n:])
        assert np.all(np.abs(budget - rb) <= TOL_FP64 * np.maximum(np.abs(rb), 1e-300)), (budget, rb)
    if "buoy_ref_level" in rec:
        assert np.max(np.abs(buoy - rec["buoy_ref_level"])) <= TOL_FP64 * np.max(np.abs(rec["buoy_ref_level"]))
