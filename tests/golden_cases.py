"""Loading and checking the golden fixtures written by tests/golden/make_golden.py."""
from __future__ import annotations

import os

import numpy as np

from atsat_gb300 import fields as F

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def check_inputs(rec, st):
    sums = np.array([float(np.nansum(st.arrays[f])) for f in range(F.NFIELDS)])
    ref = rec["input_sums"]
    scale = np.maximum(np.abs(ref), 1e-300)
    # bit-identical where the generator runs on the same libm; the tolerance absorbs an ulp of drift
    assert np.all(np.abs(sums - ref) <= 1e-12 * scale + 1e-300), "the seeded generator drifted"


def check_outputs(rec, got: dict, tol: float, label: str):
    idx = rec["index"]
    bad = []
    for key in rec:
        if not key.startswith("s_"):
            continue
        fid = int(key[2:])
        a = got[fid].ravel()
        ref_s = rec[key]
        sums = rec[f"sum_{fid}"]
        scale = sums[2] if sums[2] > 0 else 1.0
        e = float(np.nanmax(np.abs(a[idx] - ref_s))) / scale if np.isfinite(ref_s).any() else 0.0
        if not np.array_equal(np.isnan(a[idx]), np.isnan(ref_s)):
            e = np.inf
        # whole-field checks: the sum (to the field's l1 norm) and the max norm
        es = abs(float(np.sum(a)) - sums[0]) / max(sums[1], 1e-300)
        em = abs(float(np.max(np.abs(a))) - sums[2]) / scale
        if not (e <= tol and es <= tol and em <= tol):
            bad.append(f"{F.NAMES[fid]}: sample {e:.2e} sum {es:.2e} max {em:.2e}")
    assert not bad, f"{label}: " + "; ".join(bad)


def check_closure_arrays(rec, prod, vel_star, tol: float):
    """The turbulence closure's own arrays (production P_k, friction velocity) against a fixture."""
    for got, key, idx in ((np.asarray(prod).ravel(), "prod", rec["index"]),
                          (np.asarray(vel_star).ravel(), "vel_star", rec["vel_star_index"])):
        ref_s, sums = rec[key + "_s"], rec[key + "_sum"]
        scale = sums[2] if sums[2] > 0 else 1.0
        e = float(np.max(np.abs(got[idx] - ref_s))) / scale
        es = abs(float(np.sum(got)) - sums[0]) / max(sums[1], 1e-300)
        assert e <= tol and es <= tol, f"{key}: sample {e:.2e} sum {es:.2e}"
