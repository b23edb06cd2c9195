"""Field ids of the C ABI (include/atsat_dyn.h) and the cSaturnModel member each one stands for."""

PROG_NAMES = ["u", "v", "w", "t", "h2o", "h2o_cloud", "h2o_ice", "h2s", "nh3", "nh3_cloud",
              "nh3_ice", "ch4", "ch4_cloud", "ch4_ice", "nh4sh", "tke", "dis"]
NPROG = 17

(U, V, W, T, H2O, H2O_CLOUD, H2O_ICE, H2S, NH3, NH3_CLOUD, NH3_ICE, CH4, CH4_CLOUD, CH4_ICE,
 NH4SH, TKE, DIS) = range(17)
N_BASE = 17
(UN, VN, WN, TN, H2ON, H2O_CLOUDN, H2O_ICEN, H2SN, NH3N, NH3_CLOUDN, NH3_ICEN, CH4N,
 CH4_CLOUDN, CH4_ICEN, NH4SHN, TKEN, DISN) = range(17, 34)
P_DYN, P_STAT, P_METRIC, RHO_MIX = 34, 35, 36, 37
(NUE, Q_PRECIP, Q_RAD, TKE_SOURCE, DIS_SOURCE,
 S_PRECIP_H2O, S_PRECIP_H2O_CLOUD, S_PRECIP_H2O_ICE,
 S_PRECIP_NH3, S_PRECIP_NH3_CLOUD, S_PRECIP_NH3_ICE,
 S_PRECIP_CH4, S_PRECIP_CH4_CLOUD, S_PRECIP_CH4_ICE,
 MASSFLUX_H2S, MASSFLUX_NH3, MASSFLUX_NH4SH, FLUXLIM_NH4SH, THERMALMASSFLUX) = range(38, 57)
RHS_BASE = 57
(RHS_U, RHS_V, RHS_W, RHS_T, RHS_H2O, RHS_H2O_CLOUD, RHS_H2O_ICE, RHS_H2S, RHS_NH3,
 RHS_NH3_CLOUD, RHS_NH3_ICE, RHS_CH4, RHS_CH4_CLOUD, RHS_CH4_ICE, RHS_NH4SH, RHS_TKE,
 RHS_DIS) = range(57, 74)
AUX_U, AUX_V, AUX_W = 74, 75, 76
P_DYNN = 77
NFIELDS = 78

S_PRECIP_FIELDS = list(range(S_PRECIP_H2O, S_PRECIP_CH4_ICE + 1))
POINT_INPUTS = list(range(NUE, THERMALMASSFLUX + 1))
RHS_FIELDS = list(range(RHS_BASE, RHS_BASE + NPROG))
AUX_FIELDS = [AUX_U, AUX_V, AUX_W]
PROG = list(range(NPROG))
PROG_N = list(range(N_BASE, N_BASE + NPROG))

NAMES = (PROG_NAMES + [n + "n" for n in PROG_NAMES]
         + ["p_dyn", "p_stat", "p_metric", "rho_mix",
            "nue", "Q_precip", "Q_rad", "tke_source", "dis_source",
            "S_precip_h2o", "S_precip_h2o_cloud", "S_precip_h2o_ice",
            "S_precip_nh3", "S_precip_nh3_cloud", "S_precip_nh3_ice",
            "S_precip_ch4", "S_precip_ch4_cloud", "S_precip_ch4_ice",
            "massflux_h2s", "massflux_nh3", "massflux_nh4sh", "fluxlim_nh4sh", "thermalmassflux"]
         + ["rhs_" + n for n in PROG_NAMES] + ["aux_u", "aux_v", "aux_w", "p_dynn"])
assert len(NAMES) == NFIELDS
ID = {n: i for i, n in enumerate(NAMES)}

# inputs a single RK4 step reads (RungeKutta_Sat_Turb.cpp:110-387 with RHSSat)
STEP_INPUTS = PROG + PROG_N + [P_DYN, P_STAT, RHO_MIX] + POINT_INPUTS
# what the host reads back after the step (BCs, restoreVar, MCA, output and restart)
STEP_OUTPUTS = PROG + [RHS_U, RHS_V, RHS_W, AUX_U, AUX_V, AUX_W]

# atsat_dyn_params fields, in struct order: (name, ctype, default)
PARAM_DOUBLES = [
    ("re", 100000.0), ("pr", 69.0),
    ("sc_h2o", 0.61), ("sc_nh3", 0.61), ("sc_h2s", 0.94), ("sc_ch4", 0.99), ("sc_nh4sh", 0.7),
    ("u_0", 470.0), ("t_ref", 134.0), ("L_atm", 500.0), ("g", 10.0), ("omega", 0.000163),
    ("Coriolis", 1.0), ("centrifugal", 1.0), ("buoyancy", 1.0), ("chemical_reaction", 1.0),
    ("cp_mix", 0.0), ("r_mix", 0.0), ("R_mix", 0.0),
    ("dt", 0.01),
    ("metric_radius_km", 58232.0), ("sinthe_min", 0.0), ("buoy_scale", 1.0),
    ("turb_coupling", 1.0), ("rad_coupling", 0.0), ("precip_coupling", 1.0),
    ("thermal_massflux", 0.0), ("species_divu", 0.0), ("pdyn_cap", 0.2),
]
PARAM_INTS = [
    ("phi_periodic", 1), ("metric_split", 1), ("coriolis_split", 1), ("hydro_buoy", 0),
    ("nd_cor", 1), ("nd_cent", 0), ("nd_buoy", 0), ("cell_hold", 1), ("adiabatic", 1),
    ("adiabatic_rho", 1), ("turb_active", 1), ("t_limiter", 0), ("buoy_legacy", 0),
    ("chrom", 0), ("cp_h2_dyn", 0), ("print_diag", 0), ("coord_stretching", 0),
    ("press_src", 1), ("press_incr", 1), ("press_sweeps", 1), ("press_wall", 0),
    ("rigid_lid", 1), ("press_line", 0), ("press_baro", 0), ("precision", 0),
    ("bc_radius_form", 2), ("bc_bottom_form", 3), ("bc_pole_form", 1), ("bc_pole_fill", 1),
    ("bc_lid_u", 1), ("bc_top_taper", 2), ("bc_species_lid_copy", 1), ("bc_species_wall_copy", 2),
    ("local_rho", 1), ("damp_pdyn", 3), ("clamp_species", 1), ("driver_glue", 0), ("press_every_step", 0),
]
