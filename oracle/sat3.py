"""ORACLE -- TEST INFRASTRUCTURE ONLY: the restart file format of cSaturnModel::save_state / load_state
(planet/FileIO_Sat.cpp:513-665), restated in numpy to check the device's writer and reader.

Header: int32 {magic, im, jm, km, iteration}, magic "SAT3" 0x53415433 (SAT2 0x53415432, SAT1 0x53415431);
then every array as im*jm*km float64 (k fastest) in the order of restart_arrays() (FileIO_Sat.cpp:513-524)
and, for SAT2 / SAT3, restart_arrays_carried() (:535-552; S_precip_ch4 last, SAT3 only). Entries are field
ids of include/atsat_dyn.h or ("host", n) for the host-physics arrays the device does not hold.
"""
from __future__ import annotations

import numpy as np

from atsat_gb300 import fields as F

MAGIC = {1: 0x53415431, 2: 0x53415432, 3: 0x53415433}
HOST_NAMES = ["difflux_h2s", "difflux_nh3", "difflux_nh4sh", "j_h2s", "j_nh3", "j_nh4sh", "w_h2s", "w_nh3",
              "w_nh4sh", "BuoyancyForce", "PresGradForce", "Q_Sensible", "jT_h2s", "jT_nh3", "jT_nh4sh"]
MAIN = [F.T, F.U, F.V, F.W, F.ID["tn"], F.ID["un"], F.ID["vn"], F.ID["wn"],
        F.H2O, F.H2O_CLOUD, F.H2O_ICE, F.ID["h2on"], F.ID["h2o_cloudn"], F.ID["h2o_icen"],
        F.H2S, F.ID["h2sn"],
        F.NH3, F.NH3_CLOUD, F.NH3_ICE, F.ID["nh3n"], F.ID["nh3_cloudn"], F.ID["nh3_icen"],
        F.CH4, F.CH4_CLOUD, F.CH4_ICE, F.ID["ch4n"], F.ID["ch4_cloudn"], F.ID["ch4_icen"],
        F.NH4SH, F.ID["nh4shn"],
        F.P_DYN, F.P_DYNN, F.P_STAT,
        F.TKE, F.DIS, F.ID["tken"], F.ID["disn"], F.NUE]
CARRIED = [F.TKE_SOURCE, F.DIS_SOURCE, ("host", 0), ("host", 1), ("host", 2), ("host", 3), ("host", 4), ("host", 5),
           F.MASSFLUX_H2S, F.MASSFLUX_NH3, F.MASSFLUX_NH4SH, F.THERMALMASSFLUX, F.FLUXLIM_NH4SH,
           F.RHS_U, F.RHS_V, F.RHO_MIX, F.Q_PRECIP,
           F.ID["S_precip_h2o"], F.ID["S_precip_h2o_cloud"], F.ID["S_precip_h2o_ice"],
           F.ID["S_precip_nh3"], F.ID["S_precip_nh3_ice"], F.ID["S_precip_nh3_cloud"],
           F.ID["S_precip_ch4_cloud"], F.ID["S_precip_ch4_ice"],
           ("host", 6), ("host", 7), ("host", 8), ("host", 9), ("host", 10), ("host", 11), ("host", 12),
           ("host", 13), ("host", 14),
           F.ID["S_precip_ch4"]]


def order(fmt: int):
    return MAIN + (CARRIED[:34] if fmt == 2 else CARRIED if fmt == 3 else [])


def write(path, arrays: dict, host: list | None, shape, iteration: int, fmt: int = 3):
    """arrays: field id -> array of `shape`; host: 15 arrays or None (zeros)."""
    im, jm, km = shape
    with open(path, "wb") as f:
        f.write(np.array([MAGIC[fmt], im, jm, km, iteration], dtype=np.int32).tobytes())
        zero = np.zeros(shape)
        for e in order(fmt):
            a = (host[e[1]] if host is not None and host[e[1]] is not None else zero) if isinstance(e, tuple) else arrays[e]
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())


def read(path):
    """(format, shape, iteration, {field id: array}, [15 host arrays])"""
    with open(path, "rb") as f:
        hdr = np.frombuffer(f.read(20), dtype=np.int32)
        fmt = {v: k for k, v in MAGIC.items()}[int(hdr[0])]
        shape = tuple(int(x) for x in hdr[1:4])
        n = int(np.prod(shape))
        arrays, host = {}, [None] * 15
        for e in order(fmt):
            a = np.frombuffer(f.read(8 * n), dtype=np.float64).reshape(shape).copy()
            if isinstance(e, tuple):
                host[e[1]] = a
            else:
                arrays[e] = a
    return fmt, shape, int(hdr[4]), arrays, host
