"""Test infrastructure: run the reference harness (oracle/_ref/ref_harness) on a synthetic state.

Only usable where the reference was built (oracle/build_ref.py); the GPU machine has no reference
tree, and its tests use the committed golden fixtures instead.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

from atsat_gb300 import fields as F

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "ref_harness")
REF_GRID = (41, 181, 361)     # the reference's compile-time grid, planet/cSaturnModel.h:711


def available() -> bool:
    return os.path.exists(HARNESS)


def write_records(path: str, recs: dict):
    with open(path, "wb") as f:
        for name, arr in recs.items():
            a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64)).ravel()
            nb = name.encode()[:47].ljust(48, b"\0")
            f.write(nb)
            f.write(np.int64(a.size).tobytes())
            f.write(a.tobytes())


def read_records(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        name = data[pos:pos + 48].split(b"\0", 1)[0].decode()
        n = int(np.frombuffer(data, np.int64, 1, pos + 48)[0])
        out[name] = np.frombuffer(data, np.float64, n, pos + 56).copy()
        pos += 56 + 8 * n
    return out


def run(state, op: str, nsteps: int = 1, iter0: int = 1, params: dict | None = None,
        env: dict | None = None, threads: int | None = None) -> dict:
    """Run op on state (synth.State at 41x181x361). Returns {field id or name: array}."""
    g = state.grid
    assert g.shape == REF_GRID, "the reference grid is fixed at 41x181x361"
    recs = {F.NAMES[fid]: arr for fid, arr in state.arrays.items()}
    if state.cell_vbar0 is not None:
        recs["cell_vbar0"] = state.cell_vbar0
        recs["cell_ubar0"] = state.cell_ubar0
    if state.p_baro is not None:
        recs["p_baro"] = state.p_baro
    for k in ("re", "pr", "dt", "turb_active"):
        if params and k in params:
            recs["param:" + k] = [float(params[k])]
    e = dict(os.environ)
    e.update(env or {})
    if threads:
        e["OMP_NUM_THREADS"] = str(threads)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_records(fin, recs)
        subprocess.run([HARNESS, fin, fout, op, str(nsteps), str(iter0)], check=True, env=e,
                       stdout=subprocess.DEVNULL)
        raw = read_records(fout)
    out = {}
    for name, arr in raw.items():
        if name in F.ID:
            out[F.ID[name]] = arr.reshape(g.shape)
        else:
            out[name] = arr
    return out
