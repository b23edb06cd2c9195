"""Generate the golden fixtures of the dynamical core from the REFERENCE itself.

Each case runs the reference's own code (oracle/_ref/ref_harness, built from the reference sources
by oracle/build_ref.py) on a seeded synthetic state at the reference's compile-time grid
41x181x361, and stores per output field:
  - values at 512 seeded sample cells (flat indices),
  - the whole-field sum, sum of |x| and max |x|,
plus the sum of every input field, so a drifting generator is detected before any comparison.

Run here (where the reference tree exists): python tests/golden/make_golden.py
The fixtures are small .npz files; the tests regenerate the inputs with atsat_gb300.synth.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from atsat_gb300 import abi, fields as F, synth  # noqa: E402

NSAMPLE = 512

# name: (op, nsteps, seed, exercise, params override)
CASES = {
    "rhs_s1": ("rhs", 1, 1, True, {}),
    "rk_s1": ("rk", 1, 1, True, {}),
    "pressure_s1": ("pressure", 1, 1, True, {}),
    "density_s1": ("density", 1, 1, True, {}),
    "steps4_s2": ("steps", 4, 2, True, {}),
    "rk_plain_s0": ("rk", 1, 0, False, {}),
    # the pressure variants of PressureSolver.h:300-308, 502-708 (knobs set in the reference's environment)
    "pressure_line_s1": ("pressure", 1, 1, True, {"press_line": 1}),
    "pressure_baro_s1": ("pressure", 1, 1, True, {"press_baro": 1}),
    "pressure_lb3_s1": ("pressure", 1, 1, True, {"press_line": 1, "press_baro": 1, "press_sweeps": 3}),
    "steps4_lb_s2": ("steps", 4, 2, True, {"press_line": 1, "press_baro": 1}),
    # the driver's glue: the p_dyn filter (cSaturnModel.cpp:894-897) and the species floor (FileIO_Sat.cpp:716-772)
    "damp_s1": ("damp", 1, 1, True, {}),
    "damp_m1_s1": ("damp", 1, 1, True, {"damp_pdyn": 1}),
    "clamp_s3": ("clamp", 1, 3, True, {}),
    "driver4_s3": ("driver", 4, 3, True, {}),
    # Turbulence<cSaturnModel>::run (Turbulence.h:306-329); "turb:" keys are the closure's own knobs
    "turb_s1": ("turb", 1, 1, True, {}),
    "turb_kw_s1": ("turb", 1, 1, True, {"turb:model": 1}),
    "turb_ke_nf_s1": ("turb", 1, 1, True, {"turb:model": 0, "turb:turb_free": 0}),
}

# cases whose state carries planted undershoots (negative and NaN species cells) for the species floor
PLANTED = {"clamp_s3", "driver4_s3"}

# the reference reads these knobs from its environment (PressureSolver.h:174-175, 300-303)
KNOB_ENV = {"press_line": "ATSAT_PRESS_LINE", "press_baro": "ATSAT_PRESS_BAROTROPIC",
            "press_sweeps": "ATSAT_PRESS_SWEEPS", "damp_pdyn": "ATSAT_DAMP_PDYN"}


TURB_ENV = {"turb:turb_free": "ATSAT_TURB_FREE", "turb:buoy": "ATSAT_TURB_BUOY", "turb:curv": "ATSAT_TURB_CURV",
            "turb:clamp_pass": "ATSAT_TURB_CLAMP_PASS", "turb:abl_taper": "ATSAT_ABL_TAPER"}
TURB_MODEL_NAMES = {0: "k_epsilon", 1: "k_omega", 2: "k_omega_SST"}


def split_over(over):
    """(the main parameters' overrides, the closure's overrides)"""
    return ({k: v for k, v in over.items() if not k.startswith("turb:")},
            {k[5:]: v for k, v in over.items() if k.startswith("turb:")})


def reference_env(over):
    env = {}
    for k, v in over.items():
        if k == "turb:model":
            env["ATSAT_TURB_MODEL"] = TURB_MODEL_NAMES[v]
        elif k in TURB_ENV:
            env[TURB_ENV[k]] = str(v)
        else:
            env[KNOB_ENV[k]] = str(v)
    return env

OUTPUTS = {
    "rhs": F.RHS_FIELDS + F.AUX_FIELDS + [F.P_METRIC],
    "rk": F.PROG + F.RHS_FIELDS + F.AUX_FIELDS + [F.P_METRIC],
    "pressure": [F.P_DYN] + F.AUX_FIELDS + [F.RHS_U, F.RHS_V, F.RHS_W],
    "density": [F.RHO_MIX],
    "steps": F.PROG + F.PROG_N + [F.P_DYN, F.P_DYNN, F.RHO_MIX, F.P_METRIC, F.NUE] + F.AUX_FIELDS
             + [F.RHS_U, F.RHS_V, F.RHS_W],
    "damp": [F.P_DYN],
    "clamp": [F.H2O, F.H2O_CLOUD, F.H2O_ICE, F.H2S, F.NH3, F.NH3_CLOUD, F.NH3_ICE, F.CH4, F.CH4_CLOUD, F.CH4_ICE,
              F.NH4SH],
}
OUTPUTS["driver"] = OUTPUTS["steps"] + [F.TKE_SOURCE, F.DIS_SOURCE]
OUTPUTS["turb"] = [F.TKE, F.DIS, F.TKEN, F.DISN, F.NUE, F.TKE_SOURCE, F.DIS_SOURCE]


def plant_undershoots(st, seed):
    """Negative cells (scattered, and patches on both radial planes) in five species, one NaN in a sixth:
    what the species floor exists for. Seeded with the package's own generator."""
    g = st.grid
    n = g.cells
    for q, f in enumerate((F.H2O, F.NH3, F.NH4SH, F.CH4_ICE, F.H2S)):
        a = st.arrays[f]
        u = synth.uniform(seed, 500 + q, n)
        pick = u < 2000.0 / n
        flat = a.reshape(-1)
        flat[pick] = -np.abs(flat[pick]) * 0.3 - 1e-9
        a[0, 5:9, 10:20] = -1e-8
        a[-1, 7, 30] = -2e-8
    st.arrays[F.NH3_CLOUD][3, 4, 5] = np.nan
    for f in range(F.NPROG):
        st.arrays[F.N_BASE + f] = st.arrays[f].copy()
    return st


def make_state(name):
    op, nsteps, seed, exercise, over = CASES[name]
    g = synth.make_grid()
    P = abi.default_params(**split_over(over)[0])
    st = synth.saturn_state(g, P, seed=seed, exercise=exercise)
    if name in PLANTED:
        plant_undershoots(st, seed)
    return g, P, st


def sample_index(name, n_cells):
    rng = np.random.default_rng(abs(hash(name)) % (2 ** 32) if False else sum(map(ord, name)) * 7919)
    return np.sort(rng.choice(n_cells, size=NSAMPLE, replace=False))


def input_sums(st):
    return np.array([float(np.nansum(st.arrays[f])) for f in range(F.NFIELDS)])


def main(names=None):
    from oracle import refrun
    if not refrun.available():
        sys.exit("the reference harness is not built: python oracle/build_ref.py")
    for name, (op, nsteps, seed, exercise, over) in CASES.items():
        if names and name not in names:
            continue
        g, P, st = make_state(name)
        # one thread: the interior-mean reduction of PRESS_LINE then sums in loop order, as the oracle does
        out = refrun.run(st, op, nsteps=nsteps, env=reference_env(over), threads=1 if over else None)
        idx = sample_index(name, g.cells)
        rec = {"input_sums": input_sums(st), "index": idx}
        for fid in OUTPUTS[op]:
            a = out[fid].ravel()
            rec[f"s_{fid}"] = a[idx]
            rec[f"sum_{fid}"] = np.array([np.sum(a), np.sum(np.abs(a)), np.max(np.abs(a))])
        if "buoy_ref_level" in out and op in ("rhs", "rk"):
            rec["buoy_ref_level"] = out["buoy_ref_level"]
        if op == "turb":
            a = out["prod"].ravel()
            rec["prod_s"] = a[idx]
            rec["prod_sum"] = np.array([np.sum(a), np.sum(np.abs(a)), np.max(np.abs(a))])
            vs = out["vel_star"]
            vidx = sample_index(name + "/vel_star", vs.size)
            rec["vel_star_index"] = vidx
            rec["vel_star_s"] = vs[vidx]
            rec["vel_star_sum"] = np.array([np.sum(vs), np.sum(np.abs(vs)), np.max(np.abs(vs))])
        if "clamp_added" in out:
            rec["clamp_budget"] = np.concatenate([out["clamp_added"], out["clamp_cells"], out["clamp_added_bnd"],
                                                  out["clamp_cells_bnd"]])
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **rec)
        print(name, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1:])
