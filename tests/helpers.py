"""Shared test helpers: seeded cases, the comparison metric, and GPU runners over the C ABI."""
from __future__ import annotations

import numpy as np

from atsat_gb300 import abi, fields as F, synth

# parity bar of the FP64 drop-in after one step: max |gpu - oracle| / max |oracle| per field
TOL_FP64 = 1e-10


def case(shape=(9, 13, 17), seed=3, exercise=True, noise_scale=1.0, **over):
    g = synth.make_grid(*shape)
    P = abi.default_params(**over)
    st = synth.saturn_state(g, P, seed=seed, exercise=exercise, noise_scale=noise_scale)
    return g, P, st


def relerr(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| (absolute when b is identically zero); NaNs must coincide."""
    if not np.array_equal(np.isnan(a), np.isnan(b)):
        return float("inf")
    m = np.nanmax(np.abs(b)) if b.size else 0.0
    d = np.nanmax(np.abs(a - b)) if a.size else 0.0
    return float(d / m) if m > 0 else float(d)


def compare(got: dict, ref: dict, fids, tol: float, label: str = ""):
    bad = []
    worst = 0.0
    for fid in fids:
        e = relerr(got[fid], ref[fid])
        worst = max(worst, e)
        if not e <= tol:
            bad.append(f"{F.NAMES[fid]}: {e:.3e}")
    assert not bad, f"{label} fields above {tol:g}: " + ", ".join(bad)
    return worst


def plant_negatives(st, seed=0):
    """Negative cells in five species (scattered and on both radial planes) and one NaN: the undershoots
    cSaturnModel::clampNegativeSpecies floors. Any grid of at least 5 x 7 x 5."""
    g = st.grid
    rng = np.random.default_rng(seed)
    for f in (F.H2O, F.NH3, F.NH4SH, F.CH4_ICE, F.H2S):
        a = st.arrays[f]
        flat = a.reshape(-1)
        idx = rng.choice(flat.size, max(1, flat.size // 50), replace=False)
        flat[idx] = -np.abs(flat[idx]) * 0.3 - 1e-9
        a[0, 1:4, 1:4] = -1e-8
        a[-1, 2, 3] = -2e-8
    st.arrays[F.NH3_CLOUD][2, 3, 1] = np.nan
    for f in range(F.NPROG):
        st.arrays[F.N_BASE + f] = st.arrays[f].copy()
    return st
