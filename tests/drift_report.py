"""Long-run drift of the mixed-precision path against the FP64 oracle.

Runs the dycore iteration (density + pressure on even iterations, RK4, boundary conditions, restoreVar)
for `--steps` iterations on the device in mixed precision and in FP64, and in the oracle on the host,
from one seeded state with every source term exercised (k-omega and moisture sources included). Every
`--every` iterations it reports, per prognostic field and p_dyn, the max and RMS of |gpu - oracle|
normalised by max |oracle|, and the continuity residual max |div u| of the reference's iteration report
(planet/Reporting.h:372-397) for the three states.

    python tests/drift_report.py --steps 100 --every 10 [--shape 41,181,361] [--seed 2]

Prints one JSON object. Test infrastructure: the oracle is the checker.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)


def continuity_residual(g, P, u, v, w) -> float:
    """max |du/dr + 2u/rm + dv/dtheta / rm + cos / (rm sin) v + dw/dphi / (rm sin)| over
    i = 1..im-2, j = 1..jm-2, k = 1..km-2 (Reporting.h:372-397, metric radius, no polar cosine flip)."""
    R_km = P["metric_radius_km"]
    rm = g.rad_z + (R_km / P["L_atm"] - 1.0) if R_km > 0 else g.rad_z.copy()
    rm = rm[1:-1, None, None]
    sinthe = np.sin(g.the_z)[None, 1:-1, None]
    costhe = np.cos(g.the_z)[None, 1:-1, None]
    rmsin = rm * sinthe
    c = (slice(1, -1), slice(1, -1), slice(1, -1))
    dudr = (u[2:, 1:-1, 1:-1] - u[:-2, 1:-1, 1:-1]) / (2.0 * g.dr)
    dvdthe = (v[1:-1, 2:, 1:-1] - v[1:-1, :-2, 1:-1]) / (2.0 * g.dthe)
    dwdphi = (w[1:-1, 1:-1, 2:] - w[1:-1, 1:-1, :-2]) / (2.0 * g.dphi)
    res = dudr + 2.0 * u[c] / rm + dvdthe / rm + costhe / rmsin * v[c] + dwdphi / rmsin
    return float(np.max(np.abs(res)))


def drift(got, ref, fids, names):
    out = {}
    for f in fids:
        a, b = got[f], ref[f]
        m = float(np.max(np.abs(b))) or 1.0
        out[names[f]] = [float(np.max(np.abs(a - b))) / m, float(np.sqrt(np.mean((a - b) ** 2))) / m]
    return out


def run(shape=(41, 181, 361), steps=100, every=10, seed=2):
    from atsat_gb300 import dyn, fields as F
    from oracle import oracle
    from helpers import case
    g, P, st = case(shape, seed=seed, exercise=True)
    oracle.lib()                                   # build / load before the first CUDA call
    ref = st.copy()
    states = {"mixed": st.copy(), "fp64": st.copy()}
    cores = {k: dyn.Dycore(g, dict(P, precision=1 if k == "mixed" else 0)) for k in states}
    for k, d in cores.items():
        d.load_state(states[k])
    fids = F.PROG + [F.P_DYN]
    report = {"shape": list(shape), "steps": steps, "every": every, "seed": seed, "rows": []}
    t_or = t_gpu = 0.0
    for n in range(1, steps + 1):
        t0 = time.perf_counter()
        oracle.steps(ref, P, 1, iter0=n)
        t1 = time.perf_counter()
        for d in cores.values():
            d.iterate(n, 1)
        t_gpu += time.perf_counter() - t1
        t_or += t1 - t0
        if n % every == 0 or n == steps:
            row = {"step": n}
            for k, d in cores.items():
                d.download(list(range(F.NFIELDS)))
                row[k] = drift(states[k].arrays, ref.arrays, fids, F.NAMES)
            row["div_max"] = {k: continuity_residual(g, P, s.arrays[F.U], s.arrays[F.V], s.arrays[F.W])
                              for k, s in list(states.items()) + [("oracle", ref)]}
            report["rows"].append(row)
    for d in cores.values():
        d.close()
    report["seconds"] = {"oracle": t_or, "gpu_both": t_gpu}
    return report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--shape", default="41,181,361")
    ap.add_argument("--seed", type=int, default=2)
    a = ap.parse_args()
    rep = run(tuple(int(x) for x in a.shape.split(",")), a.steps, a.every, a.seed)
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
