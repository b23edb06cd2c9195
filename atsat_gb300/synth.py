"""Seeded synthetic Saturn states for the dynamical core.

There is no public dataset for this path: every workload is generated here, deterministically
from a seed, with counter-based splitmix64 streams and Box-Muller normals written out in numpy
(so the bytes do not depend on numpy's own generators).

Grid (cSaturnModel.cpp:42-52, lib/Array_1D.cpp:50-61): rad.z and the.z are running sums of dr and
dthe starting at r0 = 1 and the0 = 0, exactly as Array_1D::Coordinates builds them. For the default
41x181x361 shell dr = 0.025 and dthe = dphi = 1 deg; other shapes use dr = 1/(im-1),
dthe = pi/(jm-1), dphi = 2 pi/(km-1) over the same 500 km shell.

State ("Saturn jet state"): lat = 90 deg - theta, z_i = i * L_atm * dr km.
  w (zonal)       [400 exp(-(lat/15)^2) + 60 cos(6 lat)] m/s / u_0
  v (meridional)  N(0, 0.5) m/s / u_0
  u (radial)      N(0, 0.01) m/s / u_0
  T               134 K - 0.7 K/km z + 10 K (1 - (2 theta/pi - 1)^2) + N(0, 0.1 K), floored at the
                  configured tropopause temperature t_tropopause * t_ref (the linear profile alone
                  turns negative above z ~ 190 km of the 500 km shell); stored as T / t_ref
  p_stat          bar, hydrostatic column integral from p_ref (T_0/t_ref)^(g/(gam R_ref)) at i = 0
  h2o, nh3        mixing ratios 1e-3, 1e-4 x U[0.5, 1] x exp(-z / 100 km), stored as densities
                  q * rho_mix [kg/m3] (species are densities in the model, RHS_Sat_Turb.cpp:962)
  tke, dis        1e-3 / u_0^2 and 1e-4 L / u_0, uniform
  p_dyn           0
The n-level copies equal the live fields (the state right after restoreVar), cell_vbar0/ubar0 are
the zonal means of v and u over the km-1 distinct meridians (initCellHold, InitVariables_Sat.cpp:
1126-1139), and rho_mix is the ideal-gas density of computeMixtureDensity.

`exercise=True` adds small seeded noise to every input that is zero in the plain state (the other
species, p_dyn, nue, the source arrays, the stale rhs/aux boundary rows) so that every term of the
right-hand side and of the projection is non-zero in parity tests.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import fields as F

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def _mix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = (x ^ (x >> np.uint64(30))) * M1
        x = (x ^ (x >> np.uint64(27))) * M2
        return x ^ (x >> np.uint64(31))


def _stream_base(seed: int, stream: int) -> np.uint64:
    s = np.array([(seed * 1000003 + stream * 7919 + 1) & 0xFFFFFFFFFFFFFFFF], dtype=np.uint64)
    return _mix64(s)[0]


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from splitmix64 counter stream (seed, stream)."""
    base = _stream_base(seed, stream)
    with np.errstate(over="ignore"):
        ctr = base + (np.arange(1, n + 1, dtype=np.uint64) * GOLDEN)
    bits = _mix64(ctr) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """n standard normals, Box-Muller on pairs of the uniform stream."""
    m = (n + 1) // 2
    u = uniform(seed, stream, 2 * m)
    u1 = 1.0 - u[0::2]                      # (0, 1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2.0 * math.pi * u2), r * np.sin(2.0 * math.pi * u2)])
    return z[:n]


@dataclass
class Grid:
    im: int
    jm: int
    km: int
    dr: float
    dthe: float
    dphi: float
    rad_z: np.ndarray
    the_z: np.ndarray
    L_atm: float = 500.0

    @property
    def shape(self):
        return (self.im, self.jm, self.km)

    @property
    def cells(self) -> int:
        return self.im * self.jm * self.km

    @property
    def interior_rk(self) -> int:
        return (self.im - 2) * (self.jm - 4) * (self.km - 1)

    @property
    def interior_p(self) -> int:
        return (self.im - 2) * (self.jm - 2) * (self.km - 1)


def running_sum(n: int, z0: float, dz: float) -> np.ndarray:
    """Array_1D::Coordinates (lib/Array_1D.cpp:50-61): z[0] = z0, z[l] = z[l-1] + dz."""
    z = [0.0] * n
    z[0] = z0
    for l in range(1, n):
        z[l] = z[l - 1] + dz
    return np.array(z, dtype=np.float64)


def make_grid(im: int = 41, jm: int = 181, km: int = 361, L_atm: float = 500.0) -> Grid:
    pi180 = 180.0 / math.pi
    dr = 1.0 / (im - 1)                     # 0.025 at im = 41, the same double as the literal
    the_degree = 180.0 / (jm - 1)
    phi_degree = 360.0 / (km - 1)
    dthe = the_degree / pi180
    dphi = phi_degree / pi180
    return Grid(im, jm, km, dr, dthe, dphi, running_sum(im, 1.0, dr), running_sum(jm, 0.0, dthe),
                L_atm=L_atm)


@dataclass
class State:
    grid: Grid
    arrays: dict = field(default_factory=dict)      # field id -> (im, jm, km) float64, C order
    cell_vbar0: np.ndarray | None = None
    cell_ubar0: np.ndarray | None = None
    p_baro: np.ndarray | None = None

    def copy(self) -> "State":
        return State(self.grid, {k: v.copy() for k, v in self.arrays.items()},
                     None if self.cell_vbar0 is None else self.cell_vbar0.copy(),
                     None if self.cell_ubar0 is None else self.cell_ubar0.copy(),
                     None if self.p_baro is None else self.p_baro.copy())


def mixture_density(t: np.ndarray, p_stat: np.ndarray, t_ref: float, R_mix: float) -> np.ndarray:
    T = t * t_ref
    with np.errstate(divide="ignore", invalid="ignore"):
        rho = (p_stat * 1.0e5) / (R_mix * T)
    ok = (T > 0.0) & np.isfinite(rho) & (R_mix > 0.0)
    return np.where(ok, rho, 0.0)


def saturn_state(grid: Grid, params: dict, seed: int = 0, noise_scale: float = 1.0,
                 exercise: bool = False) -> State:
    """The seeded jet state described in the module docstring. `params` is a dict of
    atsat_dyn_params constants (u_0, t_ref, g, R_mix, L_atm, ...)."""
    im, jm, km = grid.shape
    n = grid.cells
    shp = grid.shape
    u_0 = params["u_0"]
    t_ref = params["t_ref"]
    R_mix = params["R_mix"]
    g = params["g"]
    gam, R_ref, p_ref, t_trop = 0.7, 3.89, 1.0, 0.4064

    pi180 = 180.0 / math.pi
    theta = grid.the_z[None, :, None]
    lat = 90.0 - grid.the_z * pi180
    z_km = np.arange(im, dtype=np.float64) * grid.L_atm * grid.dr
    zc = z_km[:, None, None]

    a = {}
    w_prof = (400.0 * np.exp(-(lat / 15.0) ** 2) + 60.0 * np.cos(6.0 * lat / pi180)) / u_0
    a[F.W] = np.broadcast_to(w_prof[None, :, None], shp).copy()
    a[F.V] = (0.5 * noise_scale / u_0) * normal(seed, 1, n).reshape(shp)
    a[F.U] = (0.01 * noise_scale / u_0) * normal(seed, 2, n).reshape(shp)
    T = (134.0 - 0.7 * zc + 10.0 * (1.0 - (2.0 * theta / math.pi - 1.0) ** 2)
         + 0.1 * noise_scale * normal(seed, 3, n).reshape(shp))
    T = np.maximum(T, t_trop * t_ref)
    a[F.T] = T / t_ref

    # hydrostatic p_stat [bar]: column integral up from the polytrope at the bottom plane
    p = np.empty(shp)
    p[0] = p_ref * np.power(a[F.T][0], g / (gam * R_ref))
    dz_m = grid.L_atm * grid.dr * 1.0e3
    for i in range(1, im):
        Tm = 0.5 * (T[i - 1] + T[i])
        p[i] = p[i - 1] * np.exp(-g * dz_m / (R_mix * Tm))
    a[F.P_STAT] = p
    rho = mixture_density(a[F.T], p, t_ref, R_mix)
    a[F.RHO_MIX] = rho

    decay = np.exp(-zc / 100.0)
    a[F.H2O] = 1.0e-3 * (0.5 + 0.5 * uniform(seed, 4, n).reshape(shp)) * decay * rho
    a[F.NH3] = 1.0e-4 * (0.5 + 0.5 * uniform(seed, 5, n).reshape(shp)) * decay * rho
    for f in (F.H2O_CLOUD, F.H2O_ICE, F.H2S, F.NH3_CLOUD, F.NH3_ICE, F.CH4, F.CH4_CLOUD,
              F.CH4_ICE, F.NH4SH):
        a[f] = np.zeros(shp)
    a[F.TKE] = np.full(shp, 1.0e-3 / (u_0 * u_0))
    a[F.DIS] = np.full(shp, 1.0e-4 * (grid.L_atm * 1.0e3) / u_0)
    a[F.P_DYN] = np.zeros(shp)
    a[F.P_METRIC] = np.zeros(shp)
    for f in F.POINT_INPUTS:
        a[f] = np.zeros(shp)
    for f in F.RHS_FIELDS + F.AUX_FIELDS:
        a[f] = np.zeros(shp)

    if exercise:
        s = noise_scale
        stream = 100
        def nz(scale):
            nonlocal stream
            stream += 1
            return scale * normal(seed, stream, n).reshape(shp)
        for f in (F.H2O_CLOUD, F.H2O_ICE, F.NH3_CLOUD, F.NH3_ICE, F.CH4_CLOUD, F.CH4_ICE):
            a[f] = np.abs(nz(1.0e-6 * s)) * decay
        a[F.H2S] = np.abs(nz(1.0e-5 * s)) * decay * rho
        a[F.CH4] = np.abs(nz(1.0e-4 * s)) * rho
        a[F.NH4SH] = np.abs(nz(1.0e-6 * s))
        a[F.TKE] = a[F.TKE] * (1.0 + 0.1 * nz(s))
        a[F.DIS] = a[F.DIS] * (1.0 + 0.1 * nz(s))
        a[F.P_DYN] = nz(1.0e-3 * s)
        a[F.NUE] = nz(1.0e-5 * s)              # some negative: exercises max(0, nue)
        a[F.Q_PRECIP] = nz(1.0e-2 * s)
        a[F.Q_RAD] = nz(1.0e-2 * s)
        a[F.TKE_SOURCE] = nz(1.0e-6 * s)
        a[F.DIS_SOURCE] = nz(1.0e-6 * s)
        for f in F.S_PRECIP_FIELDS:
            a[f] = nz(1.0e-6 * s)
        for f in (F.MASSFLUX_H2S, F.MASSFLUX_NH3, F.MASSFLUX_NH4SH, F.FLUXLIM_NH4SH,
                  F.THERMALMASSFLUX):
            a[f] = nz(1.0e-6 * s)
        # stale tendencies: the rows RHSSat never writes are still read by the projection
        for f in F.RHS_FIELDS + F.AUX_FIELDS:
            a[f] = nz(1.0e-3 * s)

    for f in range(F.NPROG):
        a[F.N_BASE + f] = a[f].copy()
    a[F.P_DYNN] = a[F.P_DYN].copy()

    st = State(grid, a)
    st.cell_vbar0 = a[F.V][:, :, : km - 1].sum(axis=2) / (km - 1)
    st.cell_ubar0 = a[F.U][:, :, : km - 1].sum(axis=2) / (km - 1)
    return st


def poisson_source(grid: Grid, seed: int = 7) -> np.ndarray:
    """Standalone Poisson source: zero-mean N(0,1) with a fixed seed, smoothed by a 3-point box
    filter in theta and phi (interior P cells; zero elsewhere)."""
    im, jm, km = grid.shape
    r = normal(seed, 900, grid.cells).reshape(grid.shape)
    s = r.copy()
    s[:, 1:-1, :] = (r[:, :-2, :] + r[:, 1:-1, :] + r[:, 2:, :]) / 3.0
    ring = s[:, :, : km - 1]
    ring = (np.roll(ring, 1, axis=2) + ring + np.roll(ring, -1, axis=2)) / 3.0
    s[:, :, : km - 1] = ring
    s[:, :, km - 1] = s[:, :, 0]
    out = np.zeros(grid.shape)
    out[1:-1, 1:-1, : km - 1] = s[1:-1, 1:-1, : km - 1]
    out[1:-1, 1:-1, : km - 1] -= out[1:-1, 1:-1, : km - 1].mean()
    return out
