/*
 * atsat_dyn.h -- C ABI of the GB300 dynamical core for the ATSAT Saturn model.
 *
 * The library replaces two member functions of cSaturnModel behind plain C entry points:
 *
 *   cSaturnModel::RungeKuttaSat()              planet/RungeKutta_Sat_Turb.cpp:110-387
 *     (with computeBuoyancyRefLevel :31-50, computeMetricPressure :60-108 and the per-cell
 *      right-hand side cSaturnModel::RHSSat, planet/RHS_Sat_Turb.cpp:25-1016)
 *   PressureSolver<cSaturnModel>::run()        planet/PressureSolver.h:145-766
 *     (with its model hook cSaturnModel::prepareProjectionBoundaries, planet/Pressure_Sat.cpp:78-194)
 *
 * and, as device glue for resident multi-step runs, computeMixtureDensity (Pressure_Sat.cpp:49-62),
 * restoreVar (planet/cSaturnModel.cpp:1551-1600) and the boundary passes of BC_Sat.
 *
 * Conventions
 *   - Every entry point returns an int status: ATSAT_DYN_OK (0) or a negative ATSAT_DYN_E_* code.
 *     Nothing in the library calls exit(), abort() or traps on the device. atsat_dyn_last_error()
 *     gives a one-line reason for the last failure on a handle.
 *   - A handle owns one CUDA stream and all of its device memory. A handle is not thread-safe;
 *     different handles may be driven from different threads.
 *   - Fields are bound to HOST storage, either as the reference's ragged rows (Array::x[i][j] is
 *     one row of km doubles) or as one contiguous [im][jm][km] block. upload/download copy between
 *     the bound host storage and the device copy; every compute entry point works on the device copy
 *     only and returns when the device work is complete. In the asynchronous mode (ATSAT_DYN_ASYNC=1 in
 *     the environment at create, or atsat_dyn_set_async(h, 1)) transfers and compute calls return once
 *     queued on the handle's stream: the host must call atsat_dyn_sync before it reads downloaded arrays
 *     or changes uploaded ones, and errors of the device work (a timed-out wait) surface there. Calls
 *     that hand a device result to the host (statistics, counts, restart files, autotune, solves) wait
 *     in either mode.
 *   - There is no CPU fallback: a knob value the device path does not implement makes
 *     atsat_dyn_create return ATSAT_DYN_E_UNSUPPORTED.
 */
#ifndef ATSAT_DYN_H
#define ATSAT_DYN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ATSAT_DYN_ABI_VERSION 1

/* ---- status codes ---- */
enum {
    ATSAT_DYN_OK                 =  0,
    ATSAT_DYN_E_INVALID          = -1,  /* bad argument, size or field id */
    ATSAT_DYN_E_UNSUPPORTED      = -2,  /* a knob value the device path does not implement */
    ATSAT_DYN_E_CUDA             = -3,  /* a CUDA runtime call failed */
    ATSAT_DYN_E_TIMEOUT          = -4,  /* a bounded device wait gave up */
    ATSAT_DYN_E_NONFINITE_INPUT  = -5,  /* atsat_dyn_check_finite found NaN/Inf in an input */
    ATSAT_DYN_E_NOMEM            = -6,  /* device or pinned host allocation failed */
    ATSAT_DYN_E_UNBOUND          = -7,  /* upload/download of a field with no host binding */
    ATSAT_DYN_E_TOO_LARGE        = -8   /* a grid beyond the fixed scratch of a no-allocation call */
};

/* ---- arithmetic of the step ---- */
enum {
    ATSAT_DYN_FP64  = 0,   /* plain FP64 drop-in: every operation in double */
    ATSAT_DYN_MIXED = 1    /* FP32 stencils on FP32 stage inputs; FP64 state, accumulator,
                              level-mean reductions and Poisson defect correction */
};

/* ---- field ids ----
 * The 17 prognostic fields in the order RHSSat differentiates them (RHS_Sat_Turb.cpp:137-153). */
enum {
    ATSAT_F_U = 0, ATSAT_F_V, ATSAT_F_W, ATSAT_F_T,
    ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S,
    ATSAT_F_NH3, ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE,
    ATSAT_F_CH4, ATSAT_F_CH4_CLOUD, ATSAT_F_CH4_ICE, ATSAT_F_NH4SH,
    ATSAT_F_TKE, ATSAT_F_DIS,
    ATSAT_NPROG = 17,

    /* start-of-step copies y_n (un, vn, ..., tken, disn), same order */
    ATSAT_F_N_BASE = 17,
    ATSAT_F_UN = 17, ATSAT_F_VN, ATSAT_F_WN, ATSAT_F_TN,
    ATSAT_F_H2ON, ATSAT_F_H2O_CLOUDN, ATSAT_F_H2O_ICEN, ATSAT_F_H2SN,
    ATSAT_F_NH3N, ATSAT_F_NH3_CLOUDN, ATSAT_F_NH3_ICEN,
    ATSAT_F_CH4N, ATSAT_F_CH4_CLOUDN, ATSAT_F_CH4_ICEN, ATSAT_F_NH4SHN,
    ATSAT_F_TKEN, ATSAT_F_DISN,

    /* pressures and density */
    ATSAT_F_P_DYN = 34, ATSAT_F_P_STAT, ATSAT_F_P_METRIC, ATSAT_F_RHO_MIX,

    /* point inputs of RHSSat */
    ATSAT_F_NUE = 38, ATSAT_F_Q_PRECIP, ATSAT_F_Q_RAD, ATSAT_F_TKE_SOURCE, ATSAT_F_DIS_SOURCE,
    ATSAT_F_S_PRECIP_H2O, ATSAT_F_S_PRECIP_H2O_CLOUD, ATSAT_F_S_PRECIP_H2O_ICE,
    ATSAT_F_S_PRECIP_NH3, ATSAT_F_S_PRECIP_NH3_CLOUD, ATSAT_F_S_PRECIP_NH3_ICE,
    ATSAT_F_S_PRECIP_CH4, ATSAT_F_S_PRECIP_CH4_CLOUD, ATSAT_F_S_PRECIP_CH4_ICE,
    ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH,
    ATSAT_F_FLUXLIM_NH4SH, ATSAT_F_THERMALMASSFLUX,

    /* tendencies rhs_* in prognostic order, then aux_u/v/w */
    ATSAT_F_RHS_BASE = 57,
    ATSAT_F_RHS_U = 57, ATSAT_F_RHS_V, ATSAT_F_RHS_W, ATSAT_F_RHS_T,
    ATSAT_F_RHS_H2O, ATSAT_F_RHS_H2O_CLOUD, ATSAT_F_RHS_H2O_ICE, ATSAT_F_RHS_H2S,
    ATSAT_F_RHS_NH3, ATSAT_F_RHS_NH3_CLOUD, ATSAT_F_RHS_NH3_ICE,
    ATSAT_F_RHS_CH4, ATSAT_F_RHS_CH4_CLOUD, ATSAT_F_RHS_CH4_ICE, ATSAT_F_RHS_NH4SH,
    ATSAT_F_RHS_TKE, ATSAT_F_RHS_DIS,
    ATSAT_F_AUX_U = 74, ATSAT_F_AUX_V, ATSAT_F_AUX_W,

    /* previous-iteration dynamic pressure, written by restoreVar */
    ATSAT_F_P_DYNN = 77,

    ATSAT_NFIELDS = 78
};

/* ---- grid ----
 * rad_z and the_z are cSaturnModel::rad.z and the.z as the reference builds them
 * (Array_1D::Coordinates, lib/Array_1D.cpp:50-61: a running sum of dr / dthe). The arrays are
 * copied at create time. */
typedef struct atsat_dyn_grid {
    int32_t im, jm, km;
    int32_t reserved0;
    const double* rad_z;      /* im values */
    const double* the_z;      /* jm values, colatitude in radians */
    double dr, dthe, dphi;
} atsat_dyn_grid;

/* ---- constants and resolved knobs ----
 * The constants are cSaturnModel members after LoadConfig and ThermalPropertiesSat; the knobs
 * are the ATSAT_* environment switches resolved the way the reference resolves them
 * (atsat_dyn_params_from_env does that). */
typedef struct atsat_dyn_params {
    /* model constants */
    double re, pr;
    double sc_h2o, sc_nh3, sc_h2s, sc_ch4, sc_nh4sh;
    double u_0, t_ref, L_atm, g, omega;
    double Coriolis, centrifugal, buoyancy, chemical_reaction;
    double cp_mix, r_mix, R_mix;
    double dt;
    /* real-valued knobs */
    double metric_radius_km;   /* ATSAT_METRIC_RADIUS, 58232 (cSaturnModel.h:164-169) */
    double sinthe_min;         /* ATSAT_SINTHE_MIN, 0 (cSaturnModel.h:458-465) */
    double buoy_scale;         /* ATSAT_BUOY_SCALE, 1 (RHS_Sat_Turb.cpp:268-269) */
    double turb_coupling;      /* ATSAT_TURB_COUPLING, 1 (RHS_Sat_Turb.cpp:577-578) */
    double rad_coupling;       /* ATSAT_RAD_COUPLING, 0 (RHS_Sat_Turb.cpp:611-612) */
    double precip_coupling;    /* ATSAT_PRECIP_COUPLING, 1 (RHS_Sat_Turb.cpp:645-650) */
    double thermal_massflux;   /* ATSAT_THERMAL_MASSFLUX, 0 (RHS_Sat_Turb.cpp:749-750) */
    double species_divu;       /* ATSAT_SPECIES_DIVU, 0 (RHS_Sat_Turb.cpp:979) */
    double pdyn_cap;           /* ATSAT_PDYN_CAP, 0.2 (PressureSolver.h:168) */
    /* switches, each resolved to 0 or 1 */
    int32_t phi_periodic;      /* ATSAT_BC_PHI_PERIODIC, 1 (ATPhys.h:124-129) */
    int32_t metric_split;      /* ATSAT_METRIC_SPLIT, 1 */
    int32_t coriolis_split;    /* ATSAT_CORIOLIS_SPLIT && metric_split, 1 */
    int32_t hydro_buoy;        /* ATSAT_HYDRO_BUOY && metric_split, 0 */
    int32_t nd_cor;            /* Coriolis at L/u_0 scale: ATSAT_ND_COR, else GEO_BALANCE, else NONDIM; 1 */
    int32_t nd_cent;           /* ATSAT_ND_CENT, else NONDIM; 0 */
    int32_t nd_buoy;           /* ATSAT_ND_BUOY, else NONDIM; 0 */
    int32_t cell_hold;         /* ATSAT_CELL_HOLD, else GEO_BALANCE; 1 */
    int32_t adiabatic;         /* ATSAT_ADIABATIC, 1 */
    int32_t adiabatic_rho;     /* ATSAT_ADIABATIC_RHO, 1 */
    int32_t turb_active;       /* cSaturnModel::turb_active, 1 with turb_model k_omega_SST */
    int32_t t_limiter;         /* ATSAT_T_LIMITER, 0 */
    int32_t buoy_legacy;       /* ATSAT_BUOY_LEGACY, 0 */
    int32_t chrom;             /* ATSAT_CHROM, 0 (1 is not implemented: UNSUPPORTED) */
    int32_t cp_h2_dyn;         /* ATSAT_CP_H2 / _CP_GAS in the RHS, 0 (1: UNSUPPORTED) */
    int32_t print_diag;        /* any of ATSAT_TB/UB/CWB_DIAG, 0 (1: UNSUPPORTED) */
    int32_t coord_stretching;  /* cSaturnModel::coord_stretching, 0 */
    int32_t press_src;         /* ATSAT_PRESS_SRC, 1 */
    int32_t press_incr;        /* ATSAT_PRESS_INCR, 1 (Run() sets it under GEO_BALANCE) */
    int32_t press_sweeps;      /* ATSAT_PRESS_SWEEPS, 1 (values < 1 mean 1) */
    int32_t press_wall;        /* ATSAT_PRESS_WALL, 0 (ATSAT has no solid body) */
    int32_t rigid_lid;         /* ATSAT_BC_RIGID_LID, 1 */
    int32_t press_line;        /* ATSAT_PRESS_LINE, 0 */
    int32_t press_baro;        /* ATSAT_PRESS_BAROTROPIC (effective), 0 */
    int32_t precision;         /* ATSAT_DYN_FP64 or ATSAT_DYN_MIXED */
    /* boundary conditions of BC_Sat / BoundaryConditions.h, used by atsat_dyn_boundary_conditions */
    int32_t bc_radius_form;    /* ATSAT_BC_RADIUS_COPY, 2 = Neumann (1 copy, 2 Neumann, 3 cubic, 0 cubic) */
    int32_t bc_bottom_form;    /* ATSAT_BC_BOTTOM_FORM, 3 = cubic on i = 0 (0 = as the lid) */
    int32_t bc_pole_form;      /* ATSAT_BC_POLE_COPY, 1 = copy */
    int32_t bc_pole_fill;      /* ATSAT_BC_POLE_FILL, 1 */
    int32_t bc_lid_u;          /* ATSAT_BC_LID_U (default: BC_RIGID_LID), 1 */
    int32_t bc_top_taper;      /* ATSAT_BC_TOP_TAPER, 2 */
    int32_t bc_species_lid_copy;  /* ATSAT_BC_SPECIES_LID_COPY, 1 */
    int32_t bc_species_wall_copy; /* ATSAT_BC_SPECIES_WALL_COPY, 2 (mass-fraction copy) */
    int32_t local_rho;         /* ATSAT_LOCAL_RHO, 1 (rho_at reads rho_mix) */
    /* the driver's glue around the dycore (cSaturnModel.cpp:894-897, 1101), used by atsat_dyn_damp_pdyn,
     * atsat_dyn_clamp_negative_species and, when driver_glue is 1, by atsat_dyn_iterate */
    int32_t damp_pdyn;         /* ATSAT_DAMP_PDYN, 3 under GEO_BALANCE, else 1 */
    int32_t clamp_species;     /* 1; 0 with ATSAT_NO_CLAMP */
    int32_t driver_glue;       /* 0: atsat_dyn_iterate runs the dycore sequence only; 1: also the two above */
    /* 0: atsat_dyn_iterate runs the pressure call on even iterations, as Run does (cSaturnModel.cpp:864-873);
     * 1: on every iteration (a benchmark schedule; no reference counterpart) */
    int32_t press_every_step;
    int32_t reserved[3];
} atsat_dyn_params;

/* statistics of one pressure call */
typedef struct atsat_dyn_pstats {
    int32_t sweeps;            /* red-black sweeps done */
    int32_t reserved0;
    double  src_clamped;       /* cells whose source hit +-den*PDYN_CAP or was non-finite */
    double  max_abs_update;    /* max |p_new - p_old| over the interior, last sweep */
} atsat_dyn_pstats;

/* device-side diagnostics */
typedef struct atsat_dyn_diag {
    int64_t launches;          /* kernels launched by this handle since create */
    int64_t nonfinite;         /* non-finite cells found by the last atsat_dyn_check_finite */
    int32_t timeout;           /* a bounded device wait gave up */
    int32_t tuned_from_cache;  /* 1: the stage variant and march depth came from the autotune cache */
    int32_t reserved[4];
} atsat_dyn_diag;

typedef struct atsat_dyn* atsat_dyn_t;

/* ---- set-up ---- */

/* The reference's defaults: constants of the committed configuration (cSaturnDefaults.cpp.inc,
 * cSaturnModel.h member initialisers) and every knob at its default. cp_mix, r_mix and R_mix are
 * filled with the values ChemistrySat::ThermalPropertiesSat computes from the default composition. */
int atsat_dyn_params_default(atsat_dyn_params* p);

/* Overwrite the knob fields of *p from the ATSAT_* environment variables, resolved as the reference
 * resolves them (defaults where a variable is unset). Constants are left alone. */
int atsat_dyn_params_from_env(atsat_dyn_params* p);

int  atsat_dyn_create(const atsat_dyn_grid* g, const atsat_dyn_params* p, atsat_dyn_t* out);
void atsat_dyn_destroy(atsat_dyn_t h);
const char* atsat_dyn_last_error(atsat_dyn_t h);
int  atsat_dyn_abi_version(void);

/* ---- host bindings and transfers ---- */

/* rows[i*jm + j] points to km doubles: the layout of Array::x (lib/Array.cpp:62-70). */
int atsat_dyn_bind_host_rows(atsat_dyn_t h, int32_t field, double* const* rows);
/* base points to im*jm*km doubles, k fastest. */
int atsat_dyn_bind_host_array(atsat_dyn_t h, int32_t field, double* base);
int atsat_dyn_upload(atsat_dyn_t h, const int32_t* fields, int32_t n);
int atsat_dyn_download(atsat_dyn_t h, const int32_t* fields, int32_t n);
/* Where the device addresses host memory through the CPU's page tables (Grace-Blackwell, NVLink-C2C:
 * cudaDevAttrPageableMemoryAccessUsesHostPageTables), bound fields are moved by one kernel per upload or
 * download that reads or writes the host arrays or rows in place; elsewhere by the copy engines through
 * staging buffers. On by default where available; ATSAT_HOST_DIRECT=0 in the environment at create, or
 * atsat_dyn_set_host_direct(h, 0), selects the copy engines. Setting 1 where the device cannot address
 * host memory returns ATSAT_DYN_E_UNSUPPORTED. atsat_dyn_host_direct returns 1 when `field`'s binding
 * (or, for field -1, the handle) uses the direct path, 0 when not, a negative code on error. */
int atsat_dyn_set_host_direct(atsat_dyn_t h, int32_t enable);
/* The asynchronous mode on (1) or off (0; waits for the queued work first). See the conventions above. */
int atsat_dyn_set_async(atsat_dyn_t h, int32_t enable);
int atsat_dyn_host_direct(atsat_dyn_t h, int32_t field);

/* cell_vbar0 / cell_ubar0: im*jm values or NULL (empty vectors); p_baro: im*jm*km values or NULL. */
int atsat_dyn_set_tables(atsat_dyn_t h, const double* cell_vbar0, const double* cell_ubar0,
                         const double* p_baro);
/* buoy_ref_level[im] of the last computeBuoyancyRefLevel on the device */
int atsat_dyn_get_buoy_ref_level(atsat_dyn_t h, double* out);

/* ---- the hot path ---- */

int atsat_dyn_mixture_density(atsat_dyn_t h);          /* Pressure_Sat.cpp:49-62 */
int atsat_dyn_buoyancy_ref_level(atsat_dyn_t h);       /* RungeKutta_Sat_Turb.cpp:31-50 */
int atsat_dyn_metric_pressure(atsat_dyn_t h);          /* RungeKutta_Sat_Turb.cpp:60-108 */
/* One RHSSat pass over the RK interior (RungeKutta_Sat_Turb.cpp:220-247) on the live fields:
 * writes all rhs_* and aux_u/v/w. Uses the buoyancy level and p_metric already on the device. */
int atsat_dyn_rhs(atsat_dyn_t h);
int atsat_dyn_rk4_step(atsat_dyn_t h);                 /* RungeKutta_Sat_Turb.cpp:110-387 */
int atsat_dyn_prepare_projection_boundaries(atsat_dyn_t h);   /* Pressure_Sat.cpp:78-194 */
int atsat_dyn_pressure(atsat_dyn_t h, atsat_dyn_pstats* out); /* PressureSolver.h:145-766 */

/* ---- device glue for resident multi-step runs ---- */
int atsat_dyn_restore_var(atsat_dyn_t h);              /* restoreVar(1.0), cSaturnModel.cpp:1551-1600 */
/* BC_Sat bcTheta, bcPhi, bcRadius (cSaturnModel.cpp:1091-1093; BoundaryConditions.h:150-518,
 * BC_Sat.cpp:61-179) on the dycore's fields: the 17 prognostic fields, nue, massflux_*, fluxlim_nh4sh
 * and thermalmassflux. */
int atsat_dyn_boundary_conditions(atsat_dyn_t h);
/* n iterations of the dycore part of cSaturnModel::Run, iterations iter0 .. iter0+n-1, resident on
 * the device (cSaturnModel.cpp:864-1111): on even iterations computeMixtureDensity and the pressure
 * call; then RungeKuttaSat, the boundary conditions and restoreVar. */
int atsat_dyn_iterate(atsat_dyn_t h, int32_t iter0, int32_t n);

/* The driver's glue around the dycore (cSaturnModel::Run), for runs that keep the state on the device.
 * With params.driver_glue = 1, atsat_dyn_iterate runs atsat_dyn_damp_pdyn after each pressure call and
 * atsat_dyn_clamp_negative_species after the boundary conditions, as Run does (cSaturnModel.cpp:894-897,
 * 1101). */
/* AtomUtils::damp_wiggles (lib/Utils.cpp:229-322) on one field, no surface mask: the 1-2-1 filter
 * f += strength/4 (f[-1] - 2 f + f[+1]) along k (periodic over the km-1 distinct meridians with
 * k = km-1 their copy when ATSAT_BC_PHI_PERIODIC is on), then j (clamped at the poles), then i (clamped
 * at the walls), each axis from a copy of the field, `passes` times. Uses the handle's pressure-source
 * buffer as the copy. */
int atsat_dyn_damp_wiggles(atsat_dyn_t h, int32_t field, int32_t along_i, int32_t along_j, int32_t along_k,
                           double strength, int32_t passes);
/* the p_dyn filter Run applies after each pressure call (cSaturnModel.cpp:894-897), by params.damp_pdyn:
 * 1 along i, j and k; 2 along i; 3 along i and k (the default under GEO_BALANCE); other values nothing */
int atsat_dyn_damp_pdyn(atsat_dyn_t h);
/* cSaturnModel::clampNegativeSpecies (FileIO_Sat.cpp:716-772): the 11 condensable species floored at 0
 * where !(v >= 0), NaN included; the finite amount clipped and the cells are accumulated per species,
 * and separately for the radial planes i = 0, im-1. Nothing when params.clamp_species is 0. */
int atsat_dyn_clamp_negative_species(atsat_dyn_t h);
/* the accumulated budget of the species floor since create, 11 entries each, in the order h2o,
 * h2o_cloud, h2o_ice, h2s, nh3, nh3_cloud, nh3_ice, ch4, ch4_cloud, ch4_ice, nh4sh (the reference's
 * clamp_added, clamp_cells, clamp_added_bnd, clamp_cells_bnd) */
int atsat_dyn_clamp_budget(atsat_dyn_t h, double* added, int64_t* cells, double* added_bnd, int64_t* cells_bnd);

/* ---- the turbulence closure (Turbulence<cSaturnModel>::run, planet/Turbulence.h:306-329) ----
 * Its knobs are the ATSAT_TURB_* / NUE_MAX / VEL_STAR_MAX / ABL_TAPER environment of the reference
 * (Turbulence.h:119-187, 348-352, 712-713, 812-813) and the model's constants it reads. */
enum { ATSAT_TURB_K_EPSILON = 0, ATSAT_TURB_K_OMEGA = 1, ATSAT_TURB_K_OMEGA_SST = 2 };
typedef struct atsat_dyn_turb_params {
    int32_t model;             /* ATSAT_TURB_MODEL, else the configuration's turb_model: ATSAT_TURB_K_OMEGA_SST */
    int32_t turb_free;         /* ATSAT_TURB_FREE, 1 (no wall law; uniform background k) */
    int32_t clamp_pass;        /* ATSAT_TURB_CLAMP_PASS, 1 (the floors as passes around the source loop) */
    int32_t abl_taper;         /* ATSAT_ABL_TAPER, 0 */
    int32_t curv;              /* ATSAT_TURB_CURV, 1 (curvature terms of the velocity-gradient tensor) */
    int32_t buoy;              /* ATSAT_TURB_BUOY, 3 (moist N^2 buoyancy sink of k) */
    double  k_bg;              /* ATSAT_TURB_K_BG [m2/s2], 1.0 */
    double  l_bg;              /* ATSAT_TURB_L_BG [m]; <= 0: one mean layer, L_atm / (im - 1) */
    double  nue_max_phys;      /* ATSAT_NUE_MAX [m2/s], 1e5 */
    double  vel_star_max;      /* ATSAT_VEL_STAR_MAX [m/s], sqrt(0.002) * 200 */
    double  vel_star_ref;      /* reference friction velocity [m/s], 0.4 */
    double  z_0;               /* roughness length [m], 0.1 */
    double  nue_gas;           /* kinematic viscosity of H2/He [m2/s], 1.8e-5 */
    double  abl_height;        /* boundary-layer height [m], 20000 */
    /* the condensable gases of the moist N^2 (cSaturnModel.cpp:259-266): H2O, NH3, CH4 */
    double  ep[3], lv[3], ls[3], t_0[3];
    double  reserved[4];
} atsat_dyn_turb_params;

int atsat_dyn_turb_params_default(atsat_dyn_turb_params* tp);
int atsat_dyn_turb_params_from_env(atsat_dyn_turb_params* tp);   /* the knobs above, as the reference reads them */
int atsat_dyn_set_turb_params(atsat_dyn_t h, const atsat_dyn_turb_params* tp);   /* the handle starts with the defaults */
/* Turbulence<cSaturnModel>::run on the device fields: friction velocity, the sources of the chosen closure
 * (tke_source, dis_source, nue, the production P_k), the wall condition at i = 0, the nue cap, the seam and
 * lid-corner copies; tke and dis are floored as the reference floors them. */
int atsat_dyn_turbulence(atsat_dyn_t h);
/* the closure's own arrays after the last atsat_dyn_turbulence: the production P_k (im*jm*km, contiguous,
 * k fastest) and the friction velocity u_tau (jm*km); either may be null */
int atsat_dyn_turbulence_diag(atsat_dyn_t h, double* prod, double* vel_star);

/* ---- restart files (cSaturnModel::save_state / load_state, planet/FileIO_Sat.cpp:513-665) ----
 * The reference's binary format, byte for byte: int32 header {magic, im, jm, km, iteration} with magic
 * 0x53415433 "SAT3" (0x53415431 "SAT1" without the carried arrays), then each array as im*jm*km doubles
 * (k fastest) in the order of restart_arrays() and, for SAT2 / SAT3, restart_arrays_carried(). The arrays on
 * the device are streamed from / into HBM. Fifteen carried arrays belong to the host physics and come
 * from / go to the caller's buffers (contiguous im*jm*km doubles each; a null entry is written as zeros
 * and skipped on reading), in this order: */
#define ATSAT_DYN_RESTART_NHOST 15
/* difflux_h2s, difflux_nh3, difflux_nh4sh, j_h2s, j_nh3, j_nh4sh, w_h2s, w_nh3, w_nh4sh, BuoyancyForce,
 * PresGradForce, Q_Sensible, jT_h2s, jT_nh3, jT_nh4sh */
/* write `path`; carried = 1: SAT3 (the reference's default, ATSAT_RESTART_CARRIED), 0: SAT1 */
int atsat_dyn_save_restart(atsat_dyn_t h, const char* path, int32_t iter, int32_t carried,
                           const double* const* host_arrays);
/* read `path` (SAT1, SAT2 or SAT3) into the device fields and the host buffers; writes the iteration it
 * belongs to and the format (1, 2, 3). ATSAT_DYN_E_INVALID for a missing file, a bad header, another grid or
 * a truncated file (the reference then runs from scratch). */
int atsat_dyn_load_restart(atsat_dyn_t h, const char* path, int32_t* iter, int32_t* format, double* const* host_arrays);
/* cSaturnModel::restart_state_is_clean (FileIO_Sat.cpp:676-695): 1 when every array of restart_arrays() is
 * finite everywhere (exponent bits, as the reference tests them), else 0 */
int atsat_dyn_restart_is_clean(atsat_dyn_t h, int32_t* clean);

/* ---- diagnostics and timing ---- */
int atsat_dyn_sync(atsat_dyn_t h);
int atsat_dyn_status(atsat_dyn_t h, atsat_dyn_diag* out);
/* Failure-detection test hook (no reference counterpart; the reference has no device waits). The
 * TMA-tiled stage kernels' bounded waits give up after `clocks` SM clocks instead of 2^31 (0: back to
 * 2^31); with `withhold` > 0 each block's producer leaves the last `withhold` items of its stream unissued,
 * so that the consumers' waits for them run out. A wait that gives up makes the block set a bit of the
 * device status word and return (its producer first waits, always up to 2^31 clocks, for its own copies
 * in flight); the next synchronising call returns ATSAT_DYN_E_TIMEOUT and atsat_dyn_status counts it. The
 * model state of such a step is undefined: re-upload it. clocks in [0, 2^31], withhold in [0, 8]. */
int atsat_dyn_set_wait_test(atsat_dyn_t h, int64_t clocks, int32_t withhold);
/* Count non-finite cells of a field on the device (the reference's NaN census, FileIO_Sat.cpp:418). */
int atsat_dyn_count_nonfinite(atsat_dyn_t h, int32_t field, int64_t* count);
/* Per-kernel CUDA-event timing on the handle's stream: enable, reset, and read the launch count
 * and summed milliseconds of kernel class `kclass` (ATSAT_K_*). */
enum {
    ATSAT_K_RK_STAGE = 0,   /* fused RHS + stage update (one per RK stage) */
    ATSAT_K_LEVEL_MEAN,     /* buoyancy level mean */
    ATSAT_K_METRIC_SCAN,    /* p_metric radial prefix sum */
    ATSAT_K_PRESS_SOURCE,   /* projection source + lc_old */
    ATSAT_K_PRESS_SWEEP,    /* red-black half-sweep */
    ATSAT_K_PRESS_BOUNDARY, /* Neumann planes, seam, projection boundary prep */
    ATSAT_K_GLUE,           /* density, restoreVar, boundary conditions */
    ATSAT_K_RHS,            /* standalone RHS pass */
    ATSAT_K_PREPARE,        /* mixed precision: once-per-step FP32 copies and frozen FP64 terms */
    ATSAT_K_NCLASS
};
int atsat_dyn_profile(atsat_dyn_t h, int32_t enable);
/* Profile only the kernel classes whose bit (1 << ATSAT_K_*) is set in mask (0: none); each timed launch
 * group adds two event records to the stream, so a narrow mask keeps a timed region close to unprofiled. */
int atsat_dyn_profile_classes(atsat_dyn_t h, uint32_t mask);
int atsat_dyn_profile_reset(atsat_dyn_t h);
int atsat_dyn_profile_read(atsat_dyn_t h, int32_t kclass, int64_t* launches, double* ms);
/* Wall time of the handle's stream between two marks, from CUDA events recorded on that stream:
 * timer_start records the first, timer_stop records the second, waits for it and returns the
 * elapsed milliseconds. */
int atsat_dyn_timer_start(atsat_dyn_t h);
int atsat_dyn_timer_stop(atsat_dyn_t h, double* ms);
/* Device-side pointer and row pitch (in elements) of a field's device copy. */
int atsat_dyn_device_field(atsat_dyn_t h, int32_t field, double** dptr, int64_t* pitch);

/* Write every rhs_* at the last RK stage (RHSSat writes all of them at every stage); off by default
 * because only rhs_u/v/w are read outside the step (the projection source and the restart file). */
int atsat_dyn_set_write_all_rhs(atsat_dyn_t h, int32_t on);

/* Mixed precision: which RK stage kernel runs (all compute the same arithmetic per cell).
 *   DIRECT   one thread per cell, stencils read from global memory;
 *   TILED    halo boxes of the FP32 arrays streamed into shared memory with tensor copies (needs a
 *            driver that can encode tensor maps);
 *   SPLIT*   a momentum / temperature kernel, then a tracer kernel with 1, 3 or 13 threads per cell
 *            (not with species_divu on);
 *   SPLIT_TILED  the same momentum kernel, then the tracers TMA-tiled (4 radial levels per thread);
 *   TILED2   both the momentum / temperature and the tracer kernels TMA-tiled, every input streamed;
 *   MARCH    the momentum / temperature kernel as a radial march (a block walks a run of radial levels
 *            of its theta-phi tile, one plane per stencil array and level streamed by TMA, the radial
 *            neighbours in registers), then the TMA-tiled tracer kernel.
 * The default is MARCH where available (not with species_divu on, nor without a tensor-map encoder),
 * else TILED, else DIRECT. No reference counterpart (the reference has one CPU loop nest). Setting an
 * unavailable variant returns ATSAT_DYN_E_UNSUPPORTED. */
enum {
    ATSAT_DYN_STAGE_DIRECT = 0,
    ATSAT_DYN_STAGE_TILED = 1,
    ATSAT_DYN_STAGE_SPLIT = 2,
    ATSAT_DYN_STAGE_SPLIT3 = 3,
    ATSAT_DYN_STAGE_SPLIT13 = 4,
    ATSAT_DYN_STAGE_SPLIT_TILED = 5,
    ATSAT_DYN_STAGE_TILED2 = 6,
    ATSAT_DYN_STAGE_MARCH = 7,
    ATSAT_DYN_STAGE_NVARIANT = 8
};
int atsat_dyn_set_stage_variant(atsat_dyn_t h, int32_t variant);
int atsat_dyn_get_stage_variant(atsat_dyn_t h, int32_t* variant);
/* The MARCH variant's march depth: radial levels per block (1 .. im-2; the interior levels are split into
 * runs of this length). The default fills about 1.8 waves of resident blocks; atsat_dyn_autotune tunes it.
 * Intermediate stages that stream at most 12 point arrays (the radiation, precipitation and thermal
 * mass-flux sources off) run compact rings, three blocks per SM; ATSAT_MARCH_COMPACT=0 (read once per
 * process) keeps the regular rings, two blocks per SM. */
int atsat_dyn_set_march_levels(atsat_dyn_t h, int32_t levels);
int atsat_dyn_get_march_levels(atsat_dyn_t h, int32_t* levels);
/* Time each available stage variant on this handle's grid (`reps` launches of an intermediate RK
 * stage each, CUDA events, after two untimed launches), keep the fastest and report it with the mean
 * milliseconds of every variant in ms[ATSAT_DYN_STAGE_NVARIANT] (< 0: unavailable). The stage writes
 * only scratch buffers, so the model state is unchanged. No reference counterpart. */
int atsat_dyn_autotune(atsat_dyn_t h, int32_t reps, int32_t* chosen, double* ms);
/* The autotune cache. atsat_dyn_autotune records its choice (variant and march depth) per grid, source
 * knobs and GPU model; atsat_dyn_create of a mixed-precision handle starts from the recorded choice, with
 * no timing pass (atsat_dyn_diag.tuned_from_cache). The file is $ATSAT_DYN_TUNE_CACHE, else
 * $XDG_CACHE_HOME/atsat_dyn/autotune.txt, else $HOME/.cache/atsat_dyn/autotune.txt; ATSAT_DYN_TUNE_CACHE
 * set to "", "0" or "off" disables it. One text line per key: im jm km knobs gpu version variant levels ms
 * (knobs: bit 0 turbulence, 1 radiation source, 2 precipitation source, 3 thermal mass flux; gpu: the
 * device name with blanks as '_'). get / put read and write it directly (path NULL: the file above); get
 * returns ATSAT_DYN_E_INVALID when the key is absent. Neither touches the GPU. */
int atsat_dyn_tune_cache_get(const char* path, int32_t im, int32_t jm, int32_t km, uint32_t knobs, const char* gpu,
                             int32_t* variant, int32_t* levels, double* ms);
int atsat_dyn_tune_cache_put(const char* path, int32_t im, int32_t jm, int32_t km, uint32_t knobs, const char* gpu,
                             int32_t variant, int32_t levels, double ms);

/* ---- CUDA graphs and ensembles (no reference counterpart) ----
 * graph_capture records n (even, >= 2) resident iterations starting at iter0 (the parity of iter0 fixes
 * which of them carry the pressure call) into a CUDA graph, without running them; it needs two resident
 * iterations done first (atsat_dyn_iterate) so that the mixed path's buffers are established. A replay
 * advances the state by n iterations: graph_launch enqueues `reps` replays on the handle's stream (no sync;
 * atsat_dyn_sync waits). ensemble_run replays every member's graph `reps` times, either concurrently (each
 * member on its own stream) or one member after another, and returns the device time of the whole set
 * from CUDA events (members must live on one device). */
int atsat_dyn_graph_capture(atsat_dyn_t h, int32_t iter0, int32_t n);
int atsat_dyn_graph_launch(atsat_dyn_t h, int32_t reps);
int atsat_dyn_ensemble_run(const atsat_dyn_t* members, int32_t n, int32_t reps, int32_t concurrent, double* ms);

/* ---- standalone solves of the pressure equation ----
 * The equation the reference relaxes (PressureSolver.h:318-495 with the boundary planes of :718-746):
 *   num1 (p[i+1] + p[i-1]) + num2 (p[j+1] + p[j-1]) + num3 (p[k+1] + p[k-1]) - den p = src
 * on i = 1..im-2, j = 1..jm-2, k = 0..km-2, p[0] = c43 p[1] - c13 p[2] in r and theta, periodic in phi.
 * No reference counterpart: the reference only smooths (one red-black sweep per call). Methods:
 *   SOR64 / SOR32   red-black SOR (the reference's update, over-relaxed by omega), max_iter sweeps or
 *                   until ||src - L p|| / ||src|| <= tol (checked every 200 sweeps);
 *   REFINE_SOR      FP64 defect correction, `inner` FP32 SOR sweeps per correction;
 *   DIRECT64 / 32   real DFT over phi and a block-tridiagonal solve per mode (exact up to rounding);
 *   REFINE_DIRECT   FP64 defect correction with FP32 direct inner solves, until tol or max_iter corrections.
 * Arrays are host, contiguous im x jm x km. The operator is singular (constants): results are shifted to
 * zero mean over the interior, and a source should first be made compatible by
 * atsat_dyn_poisson_project (removes its component outside the operator's range, in place). */
enum {
    ATSAT_POISSON_SOR64 = 0,
    ATSAT_POISSON_SOR32 = 1,
    ATSAT_POISSON_REFINE_SOR = 2,
    ATSAT_POISSON_DIRECT64 = 3,
    ATSAT_POISSON_DIRECT32 = 4,
    ATSAT_POISSON_REFINE_DIRECT = 5,
    ATSAT_POISSON_NMETHOD = 6
};
typedef struct atsat_dyn_poisson_stats {
    int32_t method;
    int32_t iterations;        /* sweeps (SOR), corrections (REFINE_*), 1 (DIRECT*) */
    int32_t inner;             /* inner sweeps or inner solves in total (REFINE_*) */
    int32_t converged;         /* final relative residual <= tol */
    double  rel_residual;      /* ||src - L p||_2 / ||src||_2 in FP64 */
    double  ms;                /* device time of the solve (CUDA events) */
    int32_t sweeps_per_pass;   /* SOR sweeps between grid barriers: > 1 where the FP32 sweeps run
                                  temporally blocked, 1 for the one-sweep-per-phase kernels */
    int32_t pad;
    double  sweep_ms;          /* of ms, the device time of the SOR sweep launches alone (0: no SOR) */
    double  reserved[2];
} atsat_dyn_poisson_stats;
int atsat_dyn_poisson_project(atsat_dyn_t h, double* src);
int atsat_dyn_poisson_solve(atsat_dyn_t h, int32_t method, const double* src, double* p, double tol,
                            int32_t max_iter, int32_t inner, double omega, atsat_dyn_poisson_stats* st);

/* Pinned host memory for bound arrays (cudaHostAlloc / cudaFreeHost). */
void* atsat_dyn_host_alloc(size_t bytes);
void  atsat_dyn_host_free(void* p);

/* ---- no-allocation variant ----
 * No counterpart in the reference: the reference is host code and never faces this.
 *
 * computeBuoyancyRefLevel for callers that cannot call cudaMalloc -- a host program whose pool
 * allocator owns the whole device memory, or a time-stepping loop that must not pay cudaMalloc /
 * cudaFree (and the device synchronisation they can cause) on its critical path. The caller passes
 * its own device inputs and output; the reduction's scratch is a fixed array compiled into the library
 * (192 KB of static device memory on every GPU that loads it, held until the process exits), so the call
 * allocates nothing, host or device.
 *   t, p_stat  device arrays, element (i, j, k) at (i*jm + j)*pitch + k (the layout atsat_dyn_device_field
 *              reports), pitch >= km
 *   the_z      HOST array of the jm colatitudes (cSaturnModel::the.z); sin(the_z) weights each row
 *   buoy_out   DEVICE array of im doubles: the level means
 *   stream     the CUDA stream to run on (NULL: the default stream); the call waits for it before
 *              returning
 * Limits: im <= ATSAT_DYN_NOALLOC_MAX_IM and jm <= ATSAT_DYN_NOALLOC_MAX_JM, else ATSAT_DYN_E_TOO_LARGE.
 * The call runs on the current device: t, p_stat and buoy_out must be device memory of that device (or
 * managed memory), else ATSAT_DYN_E_INVALID. It returns ATSAT_DYN_E_CUDA without launching anything when a CUDA error from
 * earlier work is already pending (and leaves that error for its owner).
 * The call cannot be captured into a CUDA graph: it copies the_z from pageable host memory and waits for
 * its stream. The first call on a device also looks up the scratch array's device address there (once per
 * device). All calls on a device share the one scratch array:
 * calls whose GPU work overlaps (different streams or host threads at once) race on it and must be
 * serialised by the caller. Each call rewrites the scratch it reads, so nothing carries over from the
 * previous call. */
#define ATSAT_DYN_NOALLOC_MAX_IM 512
#define ATSAT_DYN_NOALLOC_MAX_JM 8192
int atsat_dyn_buoyancy_ref_level_noalloc(const double* t, const double* p_stat, int64_t pitch,
                                         int32_t im, int32_t jm, int32_t km, const double* the_z,
                                         double g, double r_mix, double R_mix, double t_ref,
                                         double* buoy_out, void* stream);

/* Self-test of the library's integer-pipe float <-> double conversions (no reference counterpart): on
 * `device`, compares them bit for bit with the hardware conversions over every one of the 2^32 binary32
 * encodings (widening, and narrowing of the widened value) and over n_doubles hashed binary64 encodings
 * (narrowing; a quarter raw bit patterns, the rest with exponents around binary32's range, a third of
 * those exact rounding ties and a third one unit either side of a tie). Writes the mismatch counts;
 * both 0 means the conversions equal the hardware's on everything tested. */
int atsat_dyn_conv_selftest(int32_t device, uint64_t n_doubles, uint64_t* bad_widen, uint64_t* bad_narrow);

#ifdef __cplusplus
}
#endif

#endif /* ATSAT_DYN_H */
