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
