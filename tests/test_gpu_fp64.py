"""FP64 drop-in parity: the CUDA path through the C ABI against the oracle, on the same seeded inputs.

The bar (TOL_FP64) is 1e-10 of max|oracle| per field after one call; the oracle itself is pinned
bit for bit to the reference by test_oracle_golden.py.
"""
import numpy as np
import pytest

from atsat_gb300 import fields as F
from oracle import oracle

from helpers import TOL_FP64, case, compare

pytestmark = pytest.mark.gpu

SHAPES = [(9, 13, 17), (21, 91, 181), (10, 20, 36), (12, 40, 70)]   # the last two: odd km-1 (seam cells share a colour)
ALL = list(range(F.NFIELDS))


def run_gpu(op, g, P, st):
    from atsat_gb300 import dyn
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.set_write_all_rhs(True)
        if op == "rhs":
            d.computeBuoyancyRefLevel()
            if P["metric_split"]:
                d.computeMetricPressure()
            d.RHSSat_pass()
        elif op == "rk":
            d.RungeKuttaSat()
        elif op == "pressure":
            d.PressureSolver_run()
        elif op == "density":
            d.computeMixtureDensity()
        elif op == "prep":
            d.prepareProjectionBoundaries()
        d.download(ALL)
        buoy = d.buoy_ref_level()
    return s, buoy


def run_oracle(op, P, st):
    s = st.copy()
    buoy = None
    if op == "rhs":
        buoy = oracle.rhs(s, P)
    elif op == "rk":
        buoy = oracle.rk4_step(s, P)
    elif op == "pressure":
        oracle.pressure(s, P)
    elif op == "density":
        oracle.mixture_density(s, P)
    elif op == "prep":
        from oracle.oracle import _Call, lib, _check
        import ctypes as C
        c = _Call(s, P)
        _check(lib().orc_prepare_projection_boundaries(C.byref(c.gh.s), C.byref(c.p), c.ptrs), "prep")
    return s, buoy


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("op", ["rhs", "rk", "pressure", "density", "prep"])
def test_parity_default_knobs(shape, op):
    g, P, st = case(shape, seed=5)
    got, gb = run_gpu(op, g, P, st)
    ref, rb = run_oracle(op, P, st)
    compare(got.arrays, ref.arrays, ALL, TOL_FP64, f"{op} {shape}")
    if rb is not None:
        assert np.max(np.abs(gb - rb)) <= TOL_FP64 * np.max(np.abs(rb))


RK_VARIANTS = [
    dict(metric_split=0, coriolis_split=0),
    dict(coriolis_split=0),
    dict(turb_active=0),
    dict(nd_buoy=1, nd_cent=1),
    dict(nd_cor=0),
    dict(species_divu=0.5),
    dict(thermal_massflux=1.0),
    dict(rad_coupling=1.0),
    dict(buoy_legacy=1),
    dict(adiabatic=0),
    dict(adiabatic_rho=0),
    dict(cell_hold=0),
    dict(precip_coupling=0.0),
    dict(turb_coupling=0.0),
    dict(re=1000.0, pr=0.69),
    dict(sinthe_min=0.3),
]


@pytest.mark.parametrize("over", RK_VARIANTS, ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_rk4_knob_variants(over):
    g, P, st = case((9, 13, 17), seed=7, **over)
    got, _ = run_gpu("rk", g, P, st)
    ref, _ = run_oracle("rk", P, st)
    compare(got.arrays, ref.arrays, ALL, TOL_FP64, f"rk {over}")


P_VARIANTS = [
    dict(press_incr=0),
    dict(press_src=0),
    dict(rigid_lid=0),
    dict(press_sweeps=4),
    dict(pdyn_cap=1e-6),
    dict(press_incr=0, rigid_lid=0, press_sweeps=3),
]


@pytest.mark.parametrize("over", P_VARIANTS, ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_pressure_knob_variants(over):
    g, P, st = case((21, 91, 181), seed=9, **over)
    got, _ = run_gpu("pressure", g, P, st)
    ref, _ = run_oracle("pressure", P, st)
    compare(got.arrays, ref.arrays, ALL, TOL_FP64, f"pressure {over}")


LINE_BARO = [dict(press_line=1), dict(press_baro=1), dict(press_line=1, press_baro=1),
             dict(press_line=1, press_baro=1, press_sweeps=3)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("over", LINE_BARO, ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_pressure_line_barotropic(shape, over):
    """PRESS_LINE (radial Thomas per column, held interior mean) and PRESS_BAROTROPIC (DFT in phi +
    tridiagonal in theta per mode) against the oracle, which equals the reference bit for bit; the odd
    km-1 grids exercise the seam column solved after its partner."""
    g, P, st = case(shape, seed=21, **over)
    got, _ = run_gpu("pressure", g, P, st)
    ref, _ = run_oracle("pressure", P, st)
    compare(got.arrays, ref.arrays, ALL, TOL_FP64, f"pressure {over} {shape}")


def test_pressure_line_holds_interior_mean():
    """After a PRESS_LINE call the interior mean of p_dyn equals its value on entry (the all-Neumann
    constant, PressureSolver.h:750-755), whatever the source."""
    from atsat_gb300 import dyn
    g, P, st = case((12, 40, 70), seed=23, press_line=1, press_sweeps=2)
    p0 = st.arrays[F.P_DYN][1:-1, 1:-1, : g.km - 1].mean()
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.PressureSolver_run()
        d.download([F.P_DYN])
    p1 = s.arrays[F.P_DYN][1:-1, 1:-1, : g.km - 1].mean()
    assert abs(p1 - p0) <= 1e-12 * max(1.0, float(np.max(np.abs(s.arrays[F.P_DYN]))))


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("mode", [3, 1, 2, 0])
def test_damp_pdyn_modes(shape, mode):
    """The p_dyn filter of cSaturnModel::Run (AtomUtils::damp_wiggles along the mode's axes)."""
    from atsat_gb300 import dyn
    g, P, st = case(shape, seed=25, damp_pdyn=mode)
    ref = st.copy()
    oracle.damp_pdyn(ref, P)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.damp_pdyn()
        d.download(ALL)
    compare(s.arrays, ref.arrays, ALL, 1e-13, f"damp mode {mode} {shape}")


@pytest.mark.parametrize("axes,strength,passes", [((1, 1, 1), 1.0, 1), ((0, 1, 0), 0.5, 3), ((1, 0, 1), 2.0, 2)])
def test_damp_wiggles_generic(axes, strength, passes):
    from atsat_gb300 import dyn
    g, P, st = case((12, 40, 70), seed=27)
    ref = st.copy()
    oracle.damp_wiggles(ref, P, F.T, *axes, strength, passes)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.damp_wiggles(F.T, *axes, strength, passes)
        d.download(ALL)
    compare(s.arrays, ref.arrays, ALL, 1e-13, f"damp {axes} {strength} {passes}")


@pytest.mark.parametrize("shape", SHAPES[:2])
def test_clamp_negative_species(shape):
    from atsat_gb300 import dyn
    from helpers import plant_negatives
    g, P, st = case(shape, seed=29)
    plant_negatives(st, seed=3)
    ref = st.copy()
    rb = oracle.clamp_negative_species(ref, P)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.clampNegativeSpecies()
        d.download(ALL)
        budget = d.clamp_budget()
    for fid in ALL:
        assert np.array_equal(s.arrays[fid], ref.arrays[fid], equal_nan=True), F.NAMES[fid]
    assert np.array_equal(budget[11:22], rb[11:22]) and np.array_equal(budget[33:], rb[33:])
    assert np.allclose(budget, rb, rtol=1e-13, atol=0.0)
    assert rb[11:22].sum() > 0 and rb[33:].sum() > 0


def test_clamp_budget_is_deterministic():
    """The floor's budget is summed in a fixed order (per-block sums, then the blocks in order): two runs
    on the same state give the same bits, with most cells of a species clipped."""
    from atsat_gb300 import dyn
    g, P, st = case((21, 91, 181), seed=33)
    st.arrays[F.H2O_CLOUD][...] = -np.abs(st.arrays[F.H2O_CLOUD]) - 1e-12
    budgets = []
    for _ in range(2):
        with dyn.Dycore(g, P) as d:
            d.load_state(st.copy())
            d.clampNegativeSpecies()
            budgets.append(d.clamp_budget())
    assert np.array_equal(budgets[0], budgets[1])
    q = [F.H2O, F.H2O_CLOUD, F.H2O_ICE, F.H2S, F.NH3, F.NH3_CLOUD, F.NH3_ICE, F.CH4, F.CH4_CLOUD, F.CH4_ICE,
         F.NH4SH].index(F.H2O_CLOUD)
    assert budgets[0][11 + q] == g.cells


def test_clamp_off_with_no_clamp():
    from atsat_gb300 import dyn
    from helpers import plant_negatives
    g, P, st = case((9, 13, 17), seed=31, clamp_species=0)
    plant_negatives(st, seed=4)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.clampNegativeSpecies()
        d.download(ALL)
        assert not d.clamp_budget().any()
    for fid in ALL:
        assert np.array_equal(s.arrays[fid], st.arrays[fid], equal_nan=True)


@pytest.mark.parametrize("shape", [(9, 13, 17), (10, 20, 36)])
def test_iterate_with_driver_glue(shape):
    """Four resident iterations with the driver's glue (p_dyn filter after the pressure call, species
    floor after the boundary conditions) against the oracle's same sequence."""
    from atsat_gb300 import dyn
    from helpers import plant_negatives
    g, P, st = case(shape, seed=33, driver_glue=1)
    plant_negatives(st, seed=5)
    ref = st.copy()
    rb = np.zeros(44)
    oracle.steps(ref, P, 4, glue=True, budget=rb)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.set_write_all_rhs(True)
        d.iterate(1, 4)
        d.download(ALL)
        budget = d.clamp_budget()
    compare(s.arrays, ref.arrays, ALL, TOL_FP64, f"driver glue {shape}")
    assert np.array_equal(budget[11:22], rb[11:22])
    assert np.allclose(budget, rb, rtol=1e-9, atol=0.0)


TURB_VARIANTS = [dict(), dict(model=1), dict(model=0), dict(turb_free=0), dict(buoy=1), dict(buoy=2, curv=0),
                 dict(abl_taper=1, nue_max_phys=1e-3), dict(buoy=0, model=0, turb_free=0)]


@pytest.mark.parametrize("shape", SHAPES)
def test_turbulence_default(shape):
    """Turbulence<cSaturnModel>::run (SST, moist buoyancy sink) against the oracle, which equals the reference."""
    _turbulence_case(shape, {})


@pytest.mark.parametrize("over", TURB_VARIANTS[1:], ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_turbulence_variants(over):
    _turbulence_case((12, 40, 70), over)


def _turbulence_case(shape, over):
    from atsat_gb300 import abi, dyn
    g, P, st = case(shape, seed=35)
    tp = abi.make_turb_params(**over)
    ref = st.copy()
    rprod, rvs = oracle.turbulence(ref, P, tp)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.set_turb_params(tp)
        d.TurbulenceSat_run()
        d.download(ALL)
        prod, vs = d.turbulence_diag()
    compare(s.arrays, ref.arrays, ALL, TOL_FP64, f"turbulence {over} {shape}")
    assert np.max(np.abs(prod - rprod)) <= TOL_FP64 * max(np.max(np.abs(rprod)), 1e-300)
    assert np.max(np.abs(vs - rvs)) <= TOL_FP64 * np.max(np.abs(rvs))


def test_turbulence_clamp_pass_off_unsupported():
    from atsat_gb300 import abi, dyn
    g, P, st = case((9, 13, 17), seed=37)
    with dyn.Dycore(g, P) as d:
        with pytest.raises(dyn.DycoreError):
            d.set_turb_params(abi.make_turb_params(clamp_pass=0))


def test_pressure_clamp_count():
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=9, pdyn_cap=1e-9)
    with dyn.Dycore(g, P) as d:
        d.load_state(st.copy())
        stats = d.PressureSolver_run()
    assert stats.sweeps == 1 and stats.src_clamped > 0


def test_dropin_sequence_host_bcs():
    """Four iterations of the dycore part of cSaturnModel::Run with the device doing density,
    pressure, RK4 and restoreVar, and the host doing the boundary conditions between them -- the
    drop-in arrangement, where the driver's own BC_Sat code stays on the CPU."""
    from atsat_gb300 import dyn
    g, P, st = case((21, 91, 181), seed=13)
    ref = st.copy()
    oracle.steps(ref, P, 4)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        for it in range(1, 5):
            if it % 2 == 0:
                d.computeMixtureDensity()
                d.PressureSolver_run()
            d.RungeKuttaSat()
            d.download(ALL)
            oracle.boundary_conditions(s, P)          # the driver's host-side BC_Sat
            d.upload(ALL)
            d.restoreVar()
        d.download(ALL)
    compare(s.arrays, ref.arrays, F.PROG + F.PROG_N + [F.P_DYN, F.RHO_MIX, F.P_METRIC] + F.AUX_FIELDS,
            TOL_FP64, "4 iterations")


def test_ragged_rows_binding():
    """The reference's own storage (one row of km doubles per (i, j)) through bind_host_rows."""
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=17)
    ref, _ = run_oracle("rk", P, st)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        rows = {}
        for fid in range(F.NFIELDS):
            a = s.arrays[fid]
            rows[fid] = [np.array(a[i, j], copy=True) for i in range(g.im) for j in range(g.jm)]
            d.bind_rows(fid, rows[fid])
        d.upload(ALL)
        d.set_tables(s.cell_vbar0, s.cell_ubar0)
        d.RungeKuttaSat()
        d.download(ALL)
    got = {fid: np.stack(rows[fid]).reshape(g.shape) for fid in range(F.NFIELDS)}
    compare(got, ref.arrays, F.PROG + [F.RHS_U, F.RHS_V, F.RHS_W, F.AUX_U], TOL_FP64, "rows")


def test_nonfinite_census():
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=19)
    st.arrays[F.T][3, 4, 5] = np.nan
    st.arrays[F.T][2, 6, 1] = np.inf
    with dyn.Dycore(g, P) as d:
        d.load_state(st)
        assert d.count_nonfinite(F.T) == 2
        assert d.count_nonfinite(F.U) == 0


@pytest.mark.parametrize("over", [dict(), dict(turb_active=0), dict(bc_top_taper=1, bc_species_wall_copy=1),
                                  dict(bc_radius_form=3, bc_bottom_form=0, bc_pole_form=2, bc_pole_fill=0),
                                  dict(local_rho=0, bc_lid_u=0)],
                         ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()) or "default")
def test_device_boundary_conditions(over):
    from atsat_gb300 import dyn
    g, P, st = case((9, 13, 17), seed=23, **over)
    ref = st.copy()
    oracle.boundary_conditions(ref, P)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.boundary_conditions()
        d.download(ALL)
    # only products and sums of two or three terms: an FMA-contracted ulp is all that may differ
    compare(s.arrays, ref.arrays, ALL, 1e-13, f"bc {over}")


@pytest.mark.parametrize("shape", SHAPES)
def test_resident_iterations(shape):
    """Six iterations of the dycore loop with everything on the device (atsat_dyn_iterate)."""
    from atsat_gb300 import dyn
    g, P, st = case(shape, seed=29)
    ref = st.copy()
    oracle.steps(ref, P, 6)
    s = st.copy()
    with dyn.Dycore(g, P) as d:
        d.load_state(s)
        d.iterate(1, 6)
        d.download(ALL)
    compare(s.arrays, ref.arrays, F.PROG + F.PROG_N + [F.P_DYN, F.P_DYNN, F.RHO_MIX, F.P_METRIC, F.NUE]
            + F.AUX_FIELDS + [F.RHS_U, F.RHS_V, F.RHS_W], TOL_FP64, f"6 iterations {shape}")
