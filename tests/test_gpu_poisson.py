"""Standalone pressure-equation solves (atsat_dyn_poisson_*) against a sparse CPU solve of the same
operator (tests/poisson_ref.py): the projection onto the operator's range, the FP64 spectral direct
solve, FP64 defect correction with FP32 inner solves, and the red-black SOR sweeps."""
import numpy as np
import pytest

import poisson_ref as PR
from helpers import case

pytestmark = pytest.mark.gpu

SHAPES = [(9, 13, 17), (12, 24, 33), (10, 20, 36)]


def problem(shape):
    from atsat_gb300 import synth
    g, P, _ = case(shape, seed=3)
    A, _ = PR.matrix(g, P)
    src = synth.poisson_source(g, seed=5)
    return g, P, A, src


@pytest.mark.parametrize("shape", SHAPES)
def test_projection_and_direct64(shape):
    from atsat_gb300 import dyn
    g, P, A, src = problem(shape)
    ref_src, _ = PR.project(g, A, src)
    x = PR.solve(g, A, ref_src)
    with dyn.Dycore(g, P) as d:
        dsrc = d.poisson_project(src)
        n = g.km - 1
        # two independent solves for the left null vector (block elimination here, sparse LU there)
        assert np.max(np.abs(dsrc[1:-1, 1:-1, :n] - ref_src[1:-1, 1:-1, :n])) <= 1e-10 * np.max(np.abs(src))
        p, st = d.poisson_solve("direct64", dsrc)
    err = np.max(np.abs(PR.to_vec(g, p) - x)) / np.max(np.abs(x))
    res = PR.rel_residual(g, A, p, ref_src)
    print(f"\n{shape} direct64: err {err:.2e} residual {res:.2e} (device {st['rel_residual']:.2e}) {st['ms']:.3f} ms")
    # both are FP64 solves of an ill-conditioned operator (radial coupling 1/dr^2 against horizontal
    # couplings ~1/rm^2): agreement to ~cond * eps
    assert err <= 1e-8
    assert res <= 1e-10 and st["rel_residual"] <= 1e-10
    # boundary planes folded as the reference's solver leaves them
    assert np.allclose(p[0], 4 / 3 * p[1] - 1 / 3 * p[2], rtol=0, atol=1e-12 * np.max(np.abs(p)))
    assert np.allclose(p[:, :, -1], p[:, :, 0], rtol=0, atol=0)


@pytest.mark.parametrize("shape", SHAPES)
def test_refine_and_fp32(shape):
    """FP32 inner solves inside FP64 defect correction: the residual falls below 1e-10 or the report
    says where it stalls; the FP32-only solve is within FP32 conditioning of the FP64 one."""
    from atsat_gb300 import dyn
    g, P, A, src = problem(shape)
    with dyn.Dycore(g, P) as d:
        f = d.poisson_project(src)
        x64, _ = d.poisson_solve("direct64", f)
        x32, s32 = d.poisson_solve("direct32", f)
        xr, sr = d.poisson_solve("refine_direct", f, tol=1e-10, max_iter=30)
    scale = np.max(np.abs(x64))
    e32 = np.max(np.abs(x32 - x64)) / scale
    er = np.max(np.abs(xr - x64)) / scale
    print(f"\n{shape} direct32: err {e32:.2e} res {s32['rel_residual']:.2e}; refine: {sr['iterations']} corrections,"
          f" res {sr['rel_residual']:.2e}, err {er:.2e}")
    assert s32["rel_residual"] < 0.1        # cond(L) * eps32 is close to 1 on these grids
    assert sr["rel_residual"] <= max(1e-10, 0.5 * s32["rel_residual"])
    if sr["converged"]:
        assert er <= 1e-8


def numpy_sweeps(g, P, f, sweeps, omega=1.0):
    """The reference's red-black update (over-relaxed by omega), then the boundary fold, per sweep."""
    num1, num2, num3, den = PR.weights(g, P)
    im, jm, km = g.shape
    n = km - 1
    p = np.zeros(g.shape)
    ii, jj, kk = np.meshgrid(np.arange(1, im - 1), np.arange(1, jm - 1), np.arange(n), indexing="ij")
    for _ in range(sweeps):
        for colour in (0, 1):
            m = ((ii + jj + kk) & 1) == colour
            i, j, k = ii[m], jj[m], kk[m]
            kw, ke = (k - 1) % n, (k + 1) % n
            acc = (p[i + 1, j, k] + p[i - 1, j, k]) * num1[i, j] + (p[i, j + 1, k] + p[i, j - 1, k]) * num2[i, j] \
                + (p[i, j, ke] + p[i, j, kw]) * num3[i, j]
            p[i, j, k] = p[i, j, k] + omega * ((acc - f[i, j, k]) / den[i, j] - p[i, j, k])
        p[0] = 4 / 3 * p[1] - 1 / 3 * p[2]
        p[-1] = 4 / 3 * p[-2] - 1 / 3 * p[-3]
        p[:, 0] = 4 / 3 * p[:, 1] - 1 / 3 * p[:, 2]
        p[:, -1] = 4 / 3 * p[:, -2] - 1 / 3 * p[:, -3]
        p[:, :, -1] = p[:, :, 0]
    p -= p[1:-1, 1:-1, :n].mean()
    return p


@pytest.mark.parametrize("shape", [(9, 13, 17), (12, 24, 33), (10, 40, 121)])
def test_sor_matches_red_black_reference(shape):
    """Red-black sweeps (omega = 1, the reference's update) from p = 0 against a numpy sweep of the same
    operator: 5 sweeps, and 213 (more than one launch of the packed solver's 200-sweep runs, its packed state
    carried from one to the next); more sweeps lower the residual (slowly: the horizontal modes are weakly
    coupled), in FP64 and FP32 alike. FP32 runs the temporally blocked sweeps: one tile along phi on the two
    smaller grids, three tiles along phi and 19 along theta on 10 x 40 x 121, an odd number of passes with a
    shorter last one at 213 sweeps."""
    from atsat_gb300 import dyn
    g, P, A, src = problem(shape)
    with dyn.Dycore(g, P) as d:
        f = d.poisson_project(src)
        p_gpu, st = d.poisson_solve("sor64", f, tol=0.0, max_iter=5, omega=1.0)
        p53, _ = d.poisson_solve("sor64", f, tol=0.0, max_iter=213, omega=1.0)
        p53_32, st53_32 = d.poisson_solve("sor32", f, tol=0.0, max_iter=213, omega=1.0)
        _, st10 = d.poisson_solve("sor64", f, tol=0.0, max_iter=400, omega=1.0)
        _, st32 = d.poisson_solve("sor32", f, tol=0.0, max_iter=400, omega=1.0)
    n = g.km - 1
    c = (slice(1, -1), slice(1, -1), slice(0, n))
    p = numpy_sweeps(g, P, f, 5)
    err = np.max(np.abs(p[c] - p_gpu[c])) / np.max(np.abs(p))
    q = numpy_sweeps(g, P, f, 213)
    err53 = np.max(np.abs(q[c] - p53[c])) / np.max(np.abs(q))
    err53_32 = np.max(np.abs(q[c] - p53_32[c])) / np.max(np.abs(q))
    print(f"\n{shape} sor64 x5 / x213 vs numpy: {err:.2e} / {err53:.2e}, sor32 x213 {err53_32:.2e}; residual after"
          f" 5 / 400 sweeps {st['rel_residual']:.3e} / {st10['rel_residual']:.3e}, fp32 400 sweeps"
          f" {st32['rel_residual']:.3e}")
    assert err <= 1e-12 and err53 <= 1e-12
    assert err53_32 <= 1e-5
    assert st53_32["sweeps_per_pass"] > 1 and st["sweeps_per_pass"] == 1     # FP32 temporally blocked
    # the folded boundary planes and the seam as the reference leaves them
    assert np.allclose(p53[0], 4 / 3 * p53[1] - 1 / 3 * p53[2], rtol=0, atol=1e-12 * np.max(np.abs(p53)))
    assert np.array_equal(p53[:, :, -1], p53[:, :, 0])
    assert st10["rel_residual"] < st["rel_residual"] < 1.0
    assert abs(st32["rel_residual"] - st10["rel_residual"]) <= 1e-3 * st10["rel_residual"]


def test_sor_over_relaxed_and_refined():
    """omega = 1.2 against numpy over 60 sweeps, and FP64 defect correction around FP32 SOR sweeps (two
    corrections of 200 sweeps) runs its inner sweeps and lowers the residual."""
    from atsat_gb300 import dyn
    g, P, A, src = problem((12, 24, 33))
    with dyn.Dycore(g, P) as d:
        f = d.poisson_project(src)
        p15, _ = d.poisson_solve("sor64", f, tol=0.0, max_iter=60, omega=1.2)
        _, s32 = d.poisson_solve("sor32", f, tol=0.0, max_iter=400, omega=1.0)
        _, sr = d.poisson_solve("refine_sor", f, tol=0.0, max_iter=2, inner=200, omega=1.0)
    n = g.km - 1
    c = (slice(1, -1), slice(1, -1), slice(0, n))
    q = numpy_sweeps(g, P, f, 60, omega=1.2)
    err = np.max(np.abs(q[c] - p15[c])) / np.max(np.abs(q))
    print(f"\nomega 1.2 x60 vs numpy {err:.2e}; sor32 x400 residual {s32['rel_residual']:.3e}, refine_sor 2 x 200"
          f" {sr['rel_residual']:.3e}")
    assert err <= 1e-11
    assert sr["inner"] == 400 and sr["rel_residual"] < 1.0
