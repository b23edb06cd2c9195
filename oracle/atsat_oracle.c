/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64, OpenMP restatement of the ATSAT dynamical core, used by tests/ and bench.py's
 * CPU-baseline leg as the checker of the CUDA path. It is never linked into, called by or shipped
 * with the product library (atsat_gb300/csrc), which fails loudly when its CUDA build is missing.
 *
 * It restates, operation by operation and in the reference's evaluation order, so that on a
 * machine without FMA contraction it agrees with the reference bit for bit (build with
 * -ffp-contract=off):
 *   cSaturnModel::computeBuoyancyRefLevel   planet/RungeKutta_Sat_Turb.cpp:31-50
 *   cSaturnModel::computeMetricPressure     planet/RungeKutta_Sat_Turb.cpp:60-108
 *   cSaturnModel::RHSSat                    planet/RHS_Sat_Turb.cpp:25-1016
 *   cSaturnModel::RungeKuttaSat             planet/RungeKutta_Sat_Turb.cpp:110-387
 *   cSaturnModel::computeMixtureDensity     planet/Pressure_Sat.cpp:49-62
 *   cSaturnModel::prepareProjectionBoundaries planet/Pressure_Sat.cpp:78-194
 *   PressureSolver<cSaturnModel>::run       planet/PressureSolver.h:145-766 (pointwise sweep, and the
 *                                           PRESS_LINE / PRESS_BAROTROPIC passes of :300-316, 502-708, 750-755)
 *   cSaturnModel::restoreVar(1.0)           planet/cSaturnModel.cpp:1551-1600
 *   AtomUtils::damp_wiggles (p_dyn filter)  lib/Utils.cpp:229-322, cSaturnModel.cpp:894-897
 *   cSaturnModel::clampNegativeSpecies      planet/FileIO_Sat.cpp:716-772
 *   Turbulence<cSaturnModel>::run           planet/Turbulence.h:306-329, 335-1115
 * Parity of this file with the reference is pinned by tests/test_oracle_golden.py against
 * fixtures produced by the reference itself (oracle/ref_harness.cpp).
 *
 * Storage: each field is one contiguous [im][jm][km] block of doubles (k fastest), indexed by the
 * field ids of include/atsat_dyn.h. The reference's ragged rows hold the same numbers.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/atsat_dyn.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846   /* the value of glibc's <math.h>, which the reference uses */
#endif

typedef struct {
    int im, jm, km;
    const double *rad_z, *the_z;
    double dr, dthe, dphi;
    const atsat_dyn_params* p;
    double** f;                 /* ATSAT_NFIELDS pointers */
    const double *vbar0, *ubar0, *p_baro;
    double* buoy;               /* im */
    double* acc[ATSAT_NPROG];   /* RK4 accumulators */
} M;

#define IDX(m, i, j, k) ((((size_t)(i)) * (m)->jm + (size_t)(j)) * (m)->km + (size_t)(k))
#define X(m, fid, i, j, k) ((m)->f[fid][IDX(m, i, j, k)])

/* std::max / std::min as the reference evaluates them (NaN passes through the same way). */
static inline double smax(double a, double b) { return (a < b) ? b : a; }
static inline double smin(double a, double b) { return (b < a) ? b : a; }

/* cSaturnModel::metricRadius, cSaturnModel.h:164-169 */
static inline double metric_radius(const M* m, double r) {
    const double R_km = m->p->metric_radius_km;
    if (!(R_km > 0.0)) return r;
    return r + (R_km / m->p->L_atm - 1.0);
}

static inline int phi_wrap(int periodic, int kk, int km) {
    if (!periodic) return kk;
    const int n = km - 1;
    return kk < 0 ? kk + n : (kk >= n ? kk - n : kk);
}

typedef struct {
    double rm, rm2, exp_rm, exp_2_rm;
    double sinthe, sinthe2, costhe, cotanthe;
    double inv_rm, inv_rm2;
    double inv_rmsinthe, inv_rm2sinthe, inv_rm2sinthe2;
    double costhe_inv_rm2sinthe;
    double inv_2dr, inv_2dthe, inv_2dphi;
    double inv_dr2, inv_dthe2, inv_dphi2;
} Geo;

/* RungeKutta_Sat_Turb.cpp:223-243 */
static void make_geo(const M* m, int i, double sinthe, double costhe, Geo* g) {
    g->rm = metric_radius(m, m->rad_z[i]);
    g->rm2 = g->rm * g->rm;
    g->exp_rm = m->p->coord_stretching ? 1.0 / (g->rm + 1.0) : 1.0;
    g->exp_2_rm = g->exp_rm * g->exp_rm;
    g->sinthe = sinthe;
    g->sinthe2 = g->sinthe * g->sinthe;
    g->costhe = costhe;
    g->cotanthe = g->costhe / g->sinthe;
    g->inv_rm = 1.0 / g->rm;
    g->inv_rm2 = 1.0 / g->rm2;
    g->inv_rmsinthe = 1.0 / (g->rm * g->sinthe);
    g->inv_rm2sinthe = g->inv_rm2 / g->sinthe;
    g->inv_rm2sinthe2 = g->inv_rm2 / g->sinthe2;
    g->costhe_inv_rm2sinthe = g->costhe * g->inv_rm2sinthe;
    g->inv_2dr = 1.0 / (2.0 * m->dr);
    g->inv_2dthe = 1.0 / (2.0 * m->dthe);
    g->inv_2dphi = 1.0 / (2.0 * m->dphi);
    g->inv_dr2 = 1.0 / (m->dr * m->dr);
    g->inv_dthe2 = 1.0 / (m->dthe * m->dthe);
    g->inv_dphi2 = 1.0 / (m->dphi * m->dphi);
}

/* ---------------- RungeKutta_Sat_Turb.cpp:31-50 ---------------- */
static void buoyancy_ref_level(M* m) {
    const atsat_dyn_params* p = m->p;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < m->im; i++) {
        double sum = 0.0, wsum = 0.0;
        for (int j = 0; j < m->jm; j++) {
            const double wgt = sin(m->the_z[j]);
            for (int k = 0; k < m->km; k++) {
                const double t = X(m, ATSAT_F_T, i, j, k);
                if (!(t > 0.0)) continue;
                const double b = p->g * X(m, ATSAT_F_P_STAT, i, j, k) / (p->r_mix * p->R_mix * t * p->t_ref);
                if (!isfinite(b)) continue;
                sum += wgt * b;
                wsum += wgt;
            }
        }
        m->buoy[i] = (wsum > 0.0) ? sum / wsum : 0.0;
    }
}

/* ---------------- RungeKutta_Sat_Turb.cpp:60-108 ---------------- */
static void metric_pressure(M* m) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const int hb = p->hydro_buoy;
    const double hb_coeff = hb ? p->g * (p->L_atm * 1.0e3) / (p->u_0 * p->u_0) : 0.0;
    double* tbar = (double*)calloc((size_t)im, sizeof(double));
    if (hb) {
        for (int i = 0; i < im; i++) {
            double s = 0.0, sw = 0.0;
            for (int j = 0; j < jm; j++) {
                const double wgt = fabs(sin(m->the_z[j]));
                for (int k = 0; k < km - 1; k++) { s += wgt * X(m, ATSAT_F_T, i, j, k); sw += wgt; }
            }
            tbar[i] = (sw > 0.0) ? s / sw : 1.0;
        }
    }
    #pragma omp parallel for collapse(2) schedule(static)
    for (int j = 0; j < jm; j++) {
        for (int k = 0; k < km; k++) {
            const double cor_ = p->coriolis_split
                ? p->Coriolis * (p->nd_cor ? p->L_atm * 1.0e3 / p->u_0 : 1.0) * 2.0 * p->omega * fabs(sin(m->the_z[j]))
                : 0.0;
            double f_prev = 0.0;
            for (int i = 0; i < im; i++) {
                const double rm_ = metric_radius(m, m->rad_z[i]);
                const double exp_rm_ = p->coord_stretching ? 1.0 / (rm_ + 1.0) : 1.0;
                const double v = X(m, ATSAT_F_V, i, j, k), w = X(m, ATSAT_F_W, i, j, k);
                double f;
                if (!hb) {
                    f = ((v * v + w * w) / rm_ + cor_ * w) / exp_rm_;
                } else {
                    const double tb_ = tbar[i], t = X(m, ATSAT_F_T, i, j, k);
                    const double b_ = (tb_ > 0.0 && isfinite(t)) ? hb_coeff * (t - tb_) / tb_ : 0.0;
                    f = ((v * v + w * w) / rm_ + cor_ * w + b_) / exp_rm_;
                }
                if (i == 0) X(m, ATSAT_F_P_METRIC, 0, j, k) = 0.0;
                else X(m, ATSAT_F_P_METRIC, i, j, k) = X(m, ATSAT_F_P_METRIC, i - 1, j, k) + 0.5 * (f_prev + f) * m->dr;
                f_prev = f;
            }
            if (m->p_baro)
                for (int i = 0; i < im; i++) X(m, ATSAT_F_P_METRIC, i, j, k) += m->p_baro[IDX(m, i, j, k)];
        }
    }
    free(tbar);
}

/* ---------------- RHS_Sat_Turb.cpp:25-1016 ---------------- */

/* One transported scalar: central first and second differences in r, theta, phi
 * (RHS_Sat_Turb.cpp:133-207). */
typedef struct { double dr, d2r, dthe, d2the, dphi, d2phi; } D6;

static inline void derivs(const M* m, int fid, int i, int j, int k, int kw, int ke, const Geo* g, D6* d) {
    const double c = X(m, fid, i, j, k);
    const double rp = X(m, fid, i + 1, j, k), rmn = X(m, fid, i - 1, j, k);
    const double tp = X(m, fid, i, j + 1, k), tmn = X(m, fid, i, j - 1, k);
    const double pe = X(m, fid, i, j, ke), pw = X(m, fid, i, j, kw);
    d->dr = (rp - rmn) * g->inv_2dr * g->exp_rm;
    d->d2r = (rp - 2.0 * c + rmn) * g->inv_dr2 * g->exp_2_rm;
    d->dthe = (tp - tmn) * g->inv_2dthe;
    d->d2the = (tp - 2.0 * c + tmn) * g->inv_dthe2;
    d->dphi = (pe - pw) * g->inv_2dphi;
    d->d2phi = (pe - 2.0 * c + pw) * g->inv_dphi2;
}

static inline double transport(double u, double v, double w, const D6* d, const Geo* g) {
    return u * d->dr + v * d->dthe * g->inv_rm + w * d->dphi * g->inv_rmsinthe;
}

static inline double diffusion(const D6* d, double two_inv_rm, const Geo* g) {
    return d->d2r + d->dr * two_inv_rm + d->d2the * g->inv_rm2
         + d->dthe * g->costhe_inv_rm2sinthe + d->d2phi * g->inv_rm2sinthe2;
}

static void rhs_cell(M* m, int i, int j, int k, const Geo* g) {
    const atsat_dyn_params* p = m->p;
    const int per = p->phi_periodic;
    const int kw = phi_wrap(per, k - 1, m->km);
    const int ke = phi_wrap(per, k + 1, m->km);
    const size_t c = IDX(m, i, j, k);
    double** f = m->f;

    const double costhe = g->costhe, cotanthe = g->cotanthe;
    const double inv_rm = g->inv_rm, inv_rm2 = g->inv_rm2, inv_rmsinthe = g->inv_rmsinthe;
    const double inv_rm2sinthe = g->inv_rm2sinthe, inv_rm2sinthe2 = g->inv_rm2sinthe2;
    const double costhe_inv_rm2sinthe = g->costhe_inv_rm2sinthe;

    const double u_ijk = f[ATSAT_F_U][c], v_ijk = f[ATSAT_F_V][c], w_ijk = f[ATSAT_F_W][c];

    D6 d[ATSAT_NPROG];
    for (int q = 0; q < ATSAT_NPROG; q++) derivs(m, q, i, j, k, kw, ke, g, &d[q]);
    const double dpdr = (X(m, ATSAT_F_P_DYN, i + 1, j, k) - X(m, ATSAT_F_P_DYN, i - 1, j, k)) * g->inv_2dr * g->exp_rm;
    const double dpdthe = (X(m, ATSAT_F_P_DYN, i, j + 1, k) - X(m, ATSAT_F_P_DYN, i, j - 1, k)) * g->inv_2dthe;
    const double dpdphi = (X(m, ATSAT_F_P_DYN, i, j, ke) - X(m, ATSAT_F_P_DYN, i, j, kw)) * g->inv_2dphi;

    /* body-force scale factors, RHS_Sat_Turb.cpp:260-277 */
    const double L_m = p->L_atm * 1.0e3;
    const double nd_cor = p->nd_cor ? L_m / p->u_0 : 1.0;
    const double nd_cent = p->nd_cent ? L_m * L_m / (p->u_0 * p->u_0) : 1.0;
    const double nd_buoy = p->nd_buoy ? 1.0e5 * L_m / (p->u_0 * p->u_0) : 1.0;

    /* Coriolis, :310-321 */
    const double sinthe_true = sqrt(smax(0.0, 1.0 - costhe * costhe));
    const double Coriolis_rad = nd_cor * -2.0 * p->omega * sinthe_true * w_ijk;
    const double Coriolis_the = nd_cor * -2.0 * p->omega * costhe * w_ijk;
    double v_cor = v_ijk, u_cor = u_ijk;
    if (p->cell_hold && m->vbar0) {
        v_cor -= m->vbar0[(size_t)i * m->jm + j];
        u_cor -= m->ubar0[(size_t)i * m->jm + j];
    }
    const double Coriolis_phi = nd_cor * +2.0 * p->omega * (+costhe * v_cor + sinthe_true * u_cor);

    /* centrifugal, :349-350 */
    const double centrifugal_rad = nd_cent * p->omega * p->omega * g->rm * sinthe_true * sinthe_true;
    const double centrifugal_the = nd_cent * p->omega * p->omega * g->rm * sinthe_true * costhe;

    const double coeff_energy_p = p->u_0 * p->u_0 / (p->cp_mix * p->t_ref);

    /* adiabatic compression work, :368-378 */
    double dpstatdr = 0.0;
    if (p->adiabatic) {
        const double to_nd = 1.0 / (p->r_mix * p->u_0 * p->u_0 * 1.0e-5);
        dpstatdr = (X(m, ATSAT_F_P_STAT, i + 1, j, k) - X(m, ATSAT_F_P_STAT, i - 1, j, k)) * g->inv_2dr * g->exp_rm * to_nd;
        const double rho_l = f[ATSAT_F_RHO_MIX][c];
        if (p->adiabatic_rho && rho_l > 0.0 && isfinite(rho_l)) dpstatdr *= p->r_mix / rho_l;
    }

    const double pressure_t = coeff_energy_p * (u_ijk * (dpdr + dpstatdr)
        + v_ijk * dpdthe * inv_rm + w_ijk * dpdphi * inv_rmsinthe);
    const double transport_t = transport(u_ijk, v_ijk, w_ijk, &d[ATSAT_F_T], g);

    const double metric_on = p->metric_split ? 0.0 : 1.0;
    const double cor_rad_on = p->coriolis_split ? 0.0 : 1.0;
    const D6 *du = &d[ATSAT_F_U], *dv = &d[ATSAT_F_V], *dw = &d[ATSAT_F_W];
    const double transport_u = u_ijk * du->dr + v_ijk * du->dthe * inv_rm + w_ijk * du->dphi * inv_rmsinthe
        - metric_on * (v_ijk * v_ijk + w_ijk * w_ijk) * inv_rm;
    const double transport_v = u_ijk * dv->dr + v_ijk * dv->dthe * inv_rm + w_ijk * dv->dphi * inv_rmsinthe
        + (u_ijk * v_ijk - w_ijk * w_ijk * cotanthe) * inv_rm;
    const double transport_w = u_ijk * dw->dr + v_ijk * dw->dthe * inv_rm + w_ijk * dw->dphi * inv_rmsinthe
        + (w_ijk * u_ijk + v_ijk * w_ijk * cotanthe) * inv_rm;

    /* diffusion, :435-491 */
    const double two_inv_rm = 2.0 * inv_rm;
    const double v_metric = (1.0 + costhe / g->sinthe2) * inv_rm2;
    const double diffusion_t = diffusion(&d[ATSAT_F_T], two_inv_rm, g);
    const double diffusion_u = du->d2r + 2.0 * u_ijk * inv_rm2 + du->d2the * inv_rm2
        + 4.0 * du->dr * inv_rm + du->dthe * costhe_inv_rm2sinthe + du->d2phi * inv_rm2sinthe2;
    const double diffusion_v = dv->d2r + dv->dr * two_inv_rm + dv->d2the * inv_rm2
        + dv->dthe * costhe_inv_rm2sinthe - v_metric * v_ijk
        + dv->d2phi * inv_rm2sinthe2 + 2.0 * du->dthe * inv_rm2
        - dw->dphi * 2.0 * costhe * inv_rm2sinthe2;
    const double diffusion_w = dw->d2r + dw->dr * two_inv_rm + dw->d2the * inv_rm2
        + dw->dthe * costhe_inv_rm2sinthe - v_metric * w_ijk
        + dw->d2phi * inv_rm2sinthe2 + 2.0 * du->dphi * inv_rm2sinthe
        + dv->dphi * 2.0 * costhe * inv_rm2sinthe2;

    /* k-omega transport, :511-538 */
    if (p->turb_active) {
        const double sig_k = 0.85, sig_w = 0.5;
        const double nue_here = f[ATSAT_F_NUE][c];
        const double transport_tke = transport(u_ijk, v_ijk, w_ijk, &d[ATSAT_F_TKE], g);
        const double transport_dis = transport(u_ijk, v_ijk, w_ijk, &d[ATSAT_F_DIS], g);
        const double diffusion_tke = diffusion(&d[ATSAT_F_TKE], two_inv_rm, g);
        const double diffusion_dis = diffusion(&d[ATSAT_F_DIS], two_inv_rm, g);
        f[ATSAT_F_RHS_TKE][c] = -transport_tke + diffusion_tke * (1.0 / p->re + nue_here / sig_k) + f[ATSAT_F_TKE_SOURCE][c];
        f[ATSAT_F_RHS_DIS][c] = -transport_dis + diffusion_dis * (1.0 / p->re + nue_here / sig_w) + f[ATSAT_F_DIS_SOURCE][c];
    } else {
        f[ATSAT_F_RHS_TKE][c] = 0.0;
        f[ATSAT_F_RHS_DIS][c] = 0.0;
    }

    /* eddy coupling, :577-582 */
    const double Pr_t = 0.9;
    const double nue_c = f[ATSAT_F_NUE][c];
    const double nue_t = (p->turb_coupling != 0.0 && isfinite(nue_c)) ? p->turb_coupling * smax(0.0, nue_c) : 0.0;
    const double nue_t_s = nue_t / Pr_t;

    /* radiation, :611-629 */
    double radiation_t = 0.0;
    if (p->rad_coupling != 0.0) {
        const double rho_f = f[ATSAT_F_RHO_MIX][c];
        const double rho = (rho_f > 0.0 && isfinite(rho_f)) ? rho_f : p->r_mix;
        const double L_rad = p->L_atm * 1.0e3;
        if (rho > 0.0 && p->cp_mix > 0.0) {
            radiation_t = p->rad_coupling * f[ATSAT_F_Q_RAD][c] * L_rad / (rho * p->cp_mix * p->u_0 * p->t_ref);
            if (!isfinite(radiation_t)) radiation_t = 0.0;
            else if (radiation_t > 0.5) radiation_t = 0.5;
            else if (radiation_t < -0.5) radiation_t = -0.5;
        }
    }

    /* precipitation latent heat, :645-665 */
    const double pc = p->precip_coupling;
    double precip_t = 0.0;
    if (pc != 0.0) {
        const double L_rad = p->L_atm * 1.0e3;
        if (p->r_mix > 0.0 && p->cp_mix > 0.0) {
            precip_t = pc * f[ATSAT_F_Q_PRECIP][c] * L_rad / (p->r_mix * p->cp_mix * p->u_0 * p->t_ref);
            if (!isfinite(precip_t)) precip_t = 0.0;
            else if (precip_t > 0.5) precip_t = 0.5;
            else if (precip_t < -0.5) precip_t = -0.5;
        }
    }

    /* buoyancy anomaly, :700-714 */
    double buoyancy_u = 0.0;
    const double t_c = f[ATSAT_F_T][c];
    if (t_c > 0.0 && !p->hydro_buoy) {
        if (p->buoy_legacy) {
            buoyancy_u = +p->buoyancy * p->g * (f[ATSAT_F_P_STAT][c] + f[ATSAT_F_P_DYN][c])
                       / (p->r_mix * p->R_mix * t_c * p->t_ref);
        } else {
            buoyancy_u = -nd_buoy * p->buoy_scale * p->buoyancy
                * (p->g * f[ATSAT_F_P_STAT][c] / (p->r_mix * p->R_mix * t_c * p->t_ref) - m->buoy[i]);
        }
    }

    /* assembly, :752-937 */
    const double tmf = p->thermal_massflux;
    f[ATSAT_F_RHS_T][c] = +pressure_t - transport_t + diffusion_t / (p->re * p->pr) + diffusion_t * nue_t_s
        - tmf * p->chemical_reaction * f[ATSAT_F_THERMALMASSFLUX][c] + radiation_t + precip_t;

    f[ATSAT_F_RHS_U][c] = -dpdr + buoyancy_u - transport_u + diffusion_u / p->re + diffusion_u * nue_t
        - cor_rad_on * p->Coriolis * Coriolis_rad + p->centrifugal * centrifugal_rad;

    double dpmdthe = 0.0, dpmdphi = 0.0;
    if (p->metric_split) {
        dpmdthe = (X(m, ATSAT_F_P_METRIC, i, j + 1, k) - X(m, ATSAT_F_P_METRIC, i, j - 1, k)) * g->inv_2dthe;
        dpmdphi = (X(m, ATSAT_F_P_METRIC, i, j, ke) - X(m, ATSAT_F_P_METRIC, i, j, kw)) * g->inv_2dphi;
    }
    f[ATSAT_F_RHS_V][c] = -dpdthe * inv_rm - dpmdthe * inv_rm - transport_v + diffusion_v / p->re + diffusion_v * nue_t
        - p->Coriolis * Coriolis_the + p->centrifugal * centrifugal_the;
    f[ATSAT_F_RHS_W][c] = -dpdphi * inv_rmsinthe - dpmdphi * inv_rmsinthe - transport_w + diffusion_w / p->re
        + diffusion_w * nue_t - p->Coriolis * Coriolis_phi;

#define SPECIES(FID, SC, EXTRA) do { \
        const double tr_ = transport(u_ijk, v_ijk, w_ijk, &d[FID], g); \
        const double df_ = diffusion(&d[FID], two_inv_rm, g); \
        f[ATSAT_F_RHS_BASE + FID][c] = -tr_ + df_ / ((SC) * p->re) + df_ * nue_t_s EXTRA; \
    } while (0)
    SPECIES(ATSAT_F_CH4, p->sc_ch4, + pc * f[ATSAT_F_S_PRECIP_CH4][c]);
    SPECIES(ATSAT_F_CH4_CLOUD, p->sc_ch4, + pc * f[ATSAT_F_S_PRECIP_CH4_CLOUD][c]);
    SPECIES(ATSAT_F_CH4_ICE, p->sc_ch4, + pc * f[ATSAT_F_S_PRECIP_CH4_ICE][c]);
    SPECIES(ATSAT_F_H2O, p->sc_h2o, + pc * f[ATSAT_F_S_PRECIP_H2O][c]);
    SPECIES(ATSAT_F_H2O_CLOUD, p->sc_h2o, + pc * f[ATSAT_F_S_PRECIP_H2O_CLOUD][c]);
    SPECIES(ATSAT_F_H2O_ICE, p->sc_h2o, + pc * f[ATSAT_F_S_PRECIP_H2O_ICE][c]);
    SPECIES(ATSAT_F_H2S, p->sc_h2s, + p->chemical_reaction * f[ATSAT_F_MASSFLUX_H2S][c]);
    SPECIES(ATSAT_F_NH3, p->sc_nh3, + p->chemical_reaction * f[ATSAT_F_MASSFLUX_NH3][c] + pc * f[ATSAT_F_S_PRECIP_NH3][c]);
    SPECIES(ATSAT_F_NH3_CLOUD, p->sc_nh3, + pc * f[ATSAT_F_S_PRECIP_NH3_CLOUD][c]);
    SPECIES(ATSAT_F_NH3_ICE, p->sc_nh3, + pc * f[ATSAT_F_S_PRECIP_NH3_ICE][c]);
#undef SPECIES
    {   /* nh4sh carries the flux-limiter correction between transport and diffusion, :932-937 */
        const double tr_ = transport(u_ijk, v_ijk, w_ijk, &d[ATSAT_F_NH4SH], g);
        const double df_ = diffusion(&d[ATSAT_F_NH4SH], two_inv_rm, g);
        f[ATSAT_F_RHS_NH4SH][c] = -tr_ + f[ATSAT_F_FLUXLIM_NH4SH][c] + df_ / (p->sc_nh4sh * p->re) + df_ * nue_t_s
            + p->chemical_reaction * f[ATSAT_F_MASSFLUX_NH4SH][c];
    }

    /* flux-form species term, :979-1009 */
    if (p->species_divu != 0.0) {
        const double sd = p->species_divu * (du->dr + 2.0 * u_ijk * inv_rm + dv->dthe * inv_rm
                                             + v_ijk * cotanthe * inv_rm + dw->dphi * inv_rmsinthe);
        static const int sp[11] = { ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                                    ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                                    ATSAT_F_CH4_ICE, ATSAT_F_NH4SH };
        for (int s = 0; s < 11; s++) f[ATSAT_F_RHS_BASE + sp[s]][c] -= sd * f[sp[s]][c];
    }

    f[ATSAT_F_AUX_U][c] = f[ATSAT_F_RHS_U][c] + dpdr;
    f[ATSAT_F_AUX_V][c] = f[ATSAT_F_RHS_V][c] + dpdthe * inv_rm;
    f[ATSAT_F_AUX_W][c] = f[ATSAT_F_RHS_W][c] + dpdphi * inv_rmsinthe;
}

static void rhs_pass(M* m) {
    const int im = m->im, jm = m->jm, km = m->km;
    const int k_first = m->p->phi_periodic ? 0 : 1;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int i = 1; i < im - 1; i++) {
        for (int j = 2; j < jm - 2; j++) {
            double st = sin(m->the_z[j]);
            if (st < m->p->sinthe_min) st = m->p->sinthe_min;
            Geo g;
            make_geo(m, i, st, cos(m->the_z[j]), &g);
            for (int k = k_first; k < km - 1; k++) rhs_cell(m, i, j, k, &g);
        }
    }
}

/* ---------------- RungeKutta_Sat_Turb.cpp:110-387 ---------------- */
static void rk4_step(M* m) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    buoyancy_ref_level(m);
    if (p->metric_split) metric_pressure(m);
    const int k_first = p->phi_periodic ? 0 : 1;
    const int turb = p->turb_active;
    const double tke_max_nd = 1000.0 / (p->u_0 * p->u_0);
    const double dis_min_nd = 1.0e-10;
    const double dt = p->dt;

    for (int stage = 0; stage < 4; stage++) {
        const double c_in = (stage == 0 || stage == 1) ? 0.5 * dt : (stage == 2 ? dt : 0.0);
        const double wgt = (stage == 0 || stage == 3) ? 1.0 : 2.0;
        rhs_pass(m);
        #pragma omp parallel for collapse(2) schedule(static)
        for (int i = 1; i < im - 1; i++) {
            for (int j = 2; j < jm - 2; j++) {
                for (int k = k_first; k < km - 1; k++) {
                    const size_t c = IDX(m, i, j, k);
                    for (int q = 0; q < ATSAT_NPROG; q++) {
                        if ((q == ATSAT_F_TKE || q == ATSAT_F_DIS) && !turb) continue;
                        const double r = m->f[ATSAT_F_RHS_BASE + q][c];
                        m->acc[q][c] = (stage == 0) ? wgt * r : m->acc[q][c] + wgt * r;
                    }
                    if (stage < 3) {
                        for (int q = 0; q < ATSAT_F_TKE; q++)
                            m->f[q][c] = m->f[ATSAT_F_N_BASE + q][c] + c_in * m->f[ATSAT_F_RHS_BASE + q][c];
                        if (turb) {
                            m->f[ATSAT_F_TKE][c] = smin(smax(m->f[ATSAT_F_TKEN][c] + c_in * m->f[ATSAT_F_RHS_TKE][c], 0.0), tke_max_nd);
                            m->f[ATSAT_F_DIS][c] = smax(m->f[ATSAT_F_DISN][c] + c_in * m->f[ATSAT_F_RHS_DIS][c], dis_min_nd);
                        }
                    }
                }
            }
        }
    }

    const double sixth_dt = dt / 6.0;
    /* the t limiter reads the OLD state tn only, so it can run in the same pass */
    #pragma omp parallel for collapse(2) schedule(static)
    for (int i = 1; i < im - 1; i++) {
        for (int j = 2; j < jm - 2; j++) {
            for (int k = k_first; k < km - 1; k++) {
                const size_t c = IDX(m, i, j, k);
                const double tn = m->f[ATSAT_F_TN][c];
                double t_new = tn + sixth_dt * m->acc[ATSAT_F_T][c];
                if (p->t_limiter) {
                    double lo = tn, hi = tn;
                    const size_t nb[6] = { IDX(m, i - 1, j, k), IDX(m, i + 1, j, k), IDX(m, i, j - 1, k),
                                           IDX(m, i, j + 1, k), IDX(m, i, j, k - 1), IDX(m, i, j, k + 1) };
                    for (int q = 0; q < 6; q++) {
                        const double val = m->f[ATSAT_F_TN][nb[q]];
                        if (val < lo) lo = val;
                        if (val > hi) hi = val;
                    }
                    if (t_new < lo) t_new = lo;
                    else if (t_new > hi) t_new = hi;
                }
                m->f[ATSAT_F_T][c] = t_new;
                if (turb) {
                    m->f[ATSAT_F_TKE][c] = smin(smax(m->f[ATSAT_F_TKEN][c] + sixth_dt * m->acc[ATSAT_F_TKE][c], 0.0), tke_max_nd);
                    m->f[ATSAT_F_DIS][c] = smax(m->f[ATSAT_F_DISN][c] + sixth_dt * m->acc[ATSAT_F_DIS][c], dis_min_nd);
                }
                for (int q = 0; q < ATSAT_F_TKE; q++) {
                    if (q == ATSAT_F_T) continue;
                    m->f[q][c] = m->f[ATSAT_F_N_BASE + q][c] + sixth_dt * m->acc[q][c];
                }
            }
        }
    }
}

/* ---------------- Pressure_Sat.cpp:49-62 ---------------- */
static void mixture_density(M* m) {
    const atsat_dyn_params* p = m->p;
    const size_t n = (size_t)m->im * m->jm * m->km;
    #pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; c++) {
        const double T = m->f[ATSAT_F_T][c] * p->t_ref;
        if (!(T > 0.0) || !(p->R_mix > 0.0)) { m->f[ATSAT_F_RHO_MIX][c] = 0.0; continue; }
        const double rho = (m->f[ATSAT_F_P_STAT][c] * 1.0e5) / (p->R_mix * T);
        m->f[ATSAT_F_RHO_MIX][c] = isfinite(rho) ? rho : 0.0;
    }
}

/* ---------------- Pressure_Sat.cpp:78-194 ---------------- */
static void prepare_projection_boundaries(M* m, int rigid_lid) {
    const int im = m->im, jm = m->jm, km = m->km;
    const int per = m->p->phi_periodic;
    const int k_first = per ? 0 : 1;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int au = ATSAT_F_AUX_U, av = ATSAT_F_AUX_V, aw = ATSAT_F_AUX_W;
    const int ru = ATSAT_F_RHS_U, rv = ATSAT_F_RHS_V, rw = ATSAT_F_RHS_W;
#define CUB_R(F_, I0, A, B, C) X(m, F_, I0, j, k) = X(m, F_, C, j, k) - 3.0 * X(m, F_, B, j, k) + 3.0 * X(m, F_, A, j, k)
#define CUB_T(F_, J0, A, B, C) X(m, F_, i, J0, k) = X(m, F_, i, C, k) - 3.0 * X(m, F_, i, B, k) + 3.0 * X(m, F_, i, A, k)
    #pragma omp parallel for
    for (int j = 1; j < jm - 1; j++) {
        for (int k = k_first; k < km - 1; k++) {
            if (rigid_lid) { X(m, au, 0, j, k) = 0.0; X(m, au, im - 1, j, k) = 0.0; }
            else { CUB_R(au, 0, 1, 2, 3); CUB_R(au, im - 1, im - 2, im - 3, im - 4); }
            CUB_R(av, 0, 1, 2, 3); CUB_R(av, im - 1, im - 2, im - 3, im - 4);
            CUB_R(aw, 0, 1, 2, 3); CUB_R(aw, im - 1, im - 2, im - 3, im - 4);
            CUB_R(ru, 0, 1, 2, 3); CUB_R(ru, im - 1, im - 2, im - 3, im - 4);
            CUB_R(rv, 0, 1, 2, 3); CUB_R(rv, im - 1, im - 2, im - 3, im - 4);
            CUB_R(rw, 0, 1, 2, 3); CUB_R(rw, im - 1, im - 2, im - 3, im - 4);
        }
    }
    #pragma omp parallel for
    for (int k = k_first; k < km - 1; k++) {
        for (int i = 1; i < im - 1; i++) {
            CUB_T(au, 0, 1, 2, 3);
            X(m, av, i, 0, k) = 0.0; X(m, aw, i, 0, k) = 0.0;
            CUB_T(au, jm - 1, jm - 2, jm - 3, jm - 4);
            X(m, av, i, jm - 1, k) = 0.0; X(m, aw, i, jm - 1, k) = 0.0;
            CUB_T(ru, 0, 1, 2, 3);
            X(m, rv, i, 0, k) = 0.0; X(m, rw, i, 0, k) = 0.0;
            CUB_T(ru, jm - 1, jm - 2, jm - 3, jm - 4);
            X(m, rv, i, jm - 1, k) = 0.0; X(m, rw, i, jm - 1, k) = 0.0;
        }
    }
#undef CUB_R
#undef CUB_T
    const int six[6] = { au, av, aw, ru, rv, rw };
    #pragma omp parallel for
    for (int i = 0; i < im; i++) {
        for (int j = 0; j < jm; j++) {
            for (int s = 0; s < 6; s++) {
                if (per) { X(m, six[s], i, j, km - 1) = X(m, six[s], i, j, 0); continue; }
                double a0 = c43 * X(m, six[s], i, j, 1) - c13 * X(m, six[s], i, j, 2);
                double a1 = c43 * X(m, six[s], i, j, km - 2) - c13 * X(m, six[s], i, j, km - 3);
                X(m, six[s], i, j, 0) = a0;
                X(m, six[s], i, j, km - 1) = a1;
                X(m, six[s], i, j, 0) = X(m, six[s], i, j, km - 1) = (X(m, six[s], i, j, 0) + X(m, six[s], i, j, km - 1)) / 2.0;
            }
        }
    }
}

/* ---------------- PressureSolver.h:300-316, 502-708: the PRESS_LINE and PRESS_BAROTROPIC passes ----------------
 * Sequential sums in the reference's loop order (its OpenMP reductions agree with these at one thread). */
static double interior_mean(const M* m, int k_first) {
    double s = 0.0;
    long cnt = 0;
    for (int i = 1; i < m->im - 1; i++)
        for (int j = 1; j < m->jm - 1; j++)
            for (int k = k_first; k < m->km - 1; k++) { s += X(m, ATSAT_F_P_DYN, i, j, k); cnt++; }
    return cnt ? s / cnt : 0.0;
}

/* PressureSolver.h:502-570: per colour ((j + k) & 1), every (j, k) column relaxed exactly in r by a
 * Thomas solve with the theta / phi neighbours lagged and both radial ends folded (p0 = c43 p1 - c13 p2).
 * The columns of one colour read only the other colour's cells except across an odd periodic seam,
 * where k = 0 and k = km-2 share a colour; rows are solved in increasing k, as one thread of the
 * reference visits them. */
static void line_pass(M* m, const double* sinthe_table, const double* line_rhs, int k_first, double inv_dr2,
                      double inv_dthe2, double inv_dphi2) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km, per = p->phi_periodic;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int P = ATSAT_F_P_DYN;
    for (int colour = 0; colour < 2; colour++) {
        #pragma omp parallel
        {
            double* aa = (double*)malloc(sizeof(double) * 6 * (size_t)im);
            double *bb = aa + im, *cc = bb + im, *dd = cc + im, *cp = dd + im, *dp = cp + im;
            #pragma omp for schedule(static)
            for (int j = 1; j < jm - 1; j++) {
                for (int k = k_first; k < km - 1; k++) {
                    if (((j + k) & 1) != colour) continue;
                    const int kw = phi_wrap(per, k - 1, km), ke = phi_wrap(per, k + 1, km);
                    for (int i = 1; i < im - 1; i++) {
                        const double rm = metric_radius(m, m->rad_z[i]);
                        const double erm = p->coord_stretching ? 1.0 / (rm + 1.0) : 1.0;
                        const double num1 = erm * erm * inv_dr2;
                        const double num2 = inv_dthe2 / (rm * rm);
                        const double num3 = inv_dphi2 / (rm * rm * sinthe_table[j] * sinthe_table[j]);
                        const double acc_h = num2 * (X(m, P, i, j + 1, k) + X(m, P, i, j - 1, k))
                                           + num3 * (X(m, P, i, j, ke) + X(m, P, i, j, kw));
                        aa[i] = -num1;
                        bb[i] = 2.0 * (num1 + num2 + num3);
                        cc[i] = -num1;
                        dd[i] = acc_h - line_rhs[IDX(m, i, j, k)];
                    }
                    const int lo = 1, hi = im - 2;
                    if (hi > lo) { bb[lo] += aa[lo] * c43; cc[lo] -= aa[lo] * c13; }
                    else dd[lo] -= aa[lo] * X(m, P, lo - 1, j, k);
                    if (hi > lo) { bb[hi] += cc[hi] * c43; aa[hi] -= cc[hi] * c13; }
                    else dd[hi] -= cc[hi] * X(m, P, hi + 1, j, k);
                    cp[lo] = cc[lo] / bb[lo];
                    dp[lo] = dd[lo] / bb[lo];
                    for (int q = lo + 1; q <= hi; q++) {
                        const double dn = bb[q] - aa[q] * cp[q - 1];
                        cp[q] = cc[q] / dn;
                        dp[q] = (dd[q] - aa[q] * dp[q - 1]) / dn;
                    }
                    double x = dp[hi];
                    if (isfinite(x)) X(m, P, hi, j, k) = x;
                    for (int q = hi - 1; q >= lo; q--) {
                        x = dp[q] - cp[q] * x;
                        if (isfinite(x)) X(m, P, q, j, k) = x;
                    }
                }
            }
            free(aa);
        }
    }
}

/* PressureSolver.h:573-708: the column residual R(j, k) = sum_i (src - Lc(p)) / sum_i 1/rm^2 (the end
 * rows read as the boundary pass sets them), its real DFT over the N = km-1 meridians, per mode a
 * tridiagonal in theta (mode 0 made consistent, pinned at j = 1 and shifted to zero sin-weighted mean),
 * and the correction q(j, k) added to every level of the column. */
static double col_resid(const M* m, const double* sinthe_table, const double* line_rhs, int j, int k,
                        double A2, double inv_dr2, double inv_dthe2, double inv_dphi2) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int P = ATSAT_F_P_DYN;
    const int kw = phi_wrap(1, k - 1, km), ke = phi_wrap(1, k + 1, km);
    double s = 0.0;
    for (int i = 1; i < im - 1; i++) {
        const double rm = metric_radius(m, m->rad_z[i]);
        const double erm = p->coord_stretching ? 1.0 / (rm + 1.0) : 1.0;
        const double num1 = erm * erm * inv_dr2;
        const double num2 = inv_dthe2 / (rm * rm);
        const double num3 = inv_dphi2 / (rm * rm * sinthe_table[j] * sinthe_table[j]);
        const double pjp = (j + 1 == jm - 1) ? c43 * X(m, P, i, jm - 2, k) - c13 * X(m, P, i, jm - 3, k) : X(m, P, i, j + 1, k);
        const double pjm = (j - 1 == 0) ? c43 * X(m, P, i, 1, k) - c13 * X(m, P, i, 2, k) : X(m, P, i, j - 1, k);
        const double pip = (i + 1 == im - 1) ? c43 * X(m, P, im - 2, j, k) - c13 * X(m, P, im - 3, j, k) : X(m, P, i + 1, j, k);
        const double pim = (i - 1 == 0) ? c43 * X(m, P, 1, j, k) - c13 * X(m, P, 2, j, k) : X(m, P, i - 1, j, k);
        const double p0 = X(m, P, i, j, k);
        const double lc = num1 * (pip + pim - 2.0 * p0)
                        + num2 * (pjp + pjm - 2.0 * p0)
                        + num3 * (X(m, P, i, j, ke) + X(m, P, i, j, kw) - 2.0 * p0);
        s += line_rhs[IDX(m, i, j, k)] - lc;
    }
    return s / A2;
}

static void barotropic_pass(M* m, const double* sinthe_table, const double* line_rhs, double inv_dr2,
                            double inv_dthe2, double inv_dphi2) {
    const int im = m->im, jm = m->jm, km = m->km;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int N = km - 1, J = jm - 2, NM = N / 2;
    double A2 = 0.0;
    for (int i = 1; i < im - 1; i++) { const double rm = metric_radius(m, m->rad_z[i]); A2 += 1.0 / (rm * rm); }
    double* R = (double*)malloc(sizeof(double) * (size_t)J * N);
    #pragma omp parallel for schedule(static)
    for (int j = 1; j < jm - 1; j++)
        for (int k = 0; k < N; k++)
            R[(size_t)(j - 1) * N + k] = col_resid(m, sinthe_table, line_rhs, j, k, A2, inv_dr2, inv_dthe2, inv_dphi2);
    double* ct = (double*)malloc(sizeof(double) * (size_t)(NM + 1) * N);
    double* stb = (double*)malloc(sizeof(double) * (size_t)(NM + 1) * N);
    for (int mm = 0; mm <= NM; mm++)
        for (int k = 0; k < N; k++) {
            const double a = 2.0 * M_PI * (double)((long)mm * k % N) / N;
            ct[(size_t)mm * N + k] = cos(a);
            stb[(size_t)mm * N + k] = sin(a);
        }
    double* Ac = (double*)calloc((size_t)(NM + 1) * J, sizeof(double));
    double* As = (double*)calloc((size_t)(NM + 1) * J, sizeof(double));
    #pragma omp parallel for collapse(2) schedule(static)
    for (int mm = 0; mm <= NM; mm++)
        for (int jj = 0; jj < J; jj++) {
            double sc = 0.0, ss = 0.0;
            const double* r_ = &R[(size_t)jj * N];
            for (int k = 0; k < N; k++) { sc += r_[k] * ct[(size_t)mm * N + k]; ss += r_[k] * stb[(size_t)mm * N + k]; }
            if (mm > 0) {
                double ra = 0.0;
                for (int k = 0; k < N; k++) ra += fabs(r_[k]);
                const double tol = 1.0e-12 * ra;
                if (fabs(sc) < tol) sc = 0.0;
                if (fabs(ss) < tol) ss = 0.0;
            }
            Ac[(size_t)mm * J + jj] = sc;
            As[(size_t)mm * J + jj] = ss;
        }
    const double e = inv_dthe2;
    #pragma omp parallel
    {
        double* a = (double*)malloc(sizeof(double) * 5 * (size_t)J);
        double *b = a + J, *c = b + J, *cp = c + J, *dp = cp + J;
        #pragma omp for schedule(static)
        for (int mm = 0; mm <= NM; mm++) {
            const double sl = sin(M_PI * mm / N);
            const double lam = 4.0 * sl * sl * inv_dphi2;
            for (int jj = 0; jj < J; jj++) {
                const double s_ = sinthe_table[jj + 1];
                a[jj] = e; c[jj] = e; b[jj] = -2.0 * e - lam / (s_ * s_);
            }
            a[0] = 0.0;     b[0] += c43 * e;     c[0] -= c13 * e;
            c[J - 1] = 0.0; b[J - 1] += c43 * e; a[J - 1] -= c13 * e;
            for (int part = 0; part < 2; part++) {
                if (mm == 0 && part == 1) continue;
                if (2 * mm == N && part == 1) continue;
                double* d = (part == 0 ? &Ac[(size_t)mm * J] : &As[(size_t)mm * J]);
                double b0 = b[0], c0 = c[0];
                if (mm == 0) {
                    double yr = 0.0, ys = 0.0;
                    for (int jj = 0; jj < J; jj++) {
                        const double y = (jj == 0 || jj == J - 1) ? 1.5 : 1.0;
                        const double s_ = fabs(sin(m->the_z[jj + 1]));
                        yr += y * d[jj]; ys += y * s_;
                    }
                    for (int jj = 0; jj < J; jj++) d[jj] -= yr / ys * fabs(sin(m->the_z[jj + 1]));
                    b0 = 1.0; c0 = 0.0; d[0] = 0.0;
                }
                cp[0] = c0 / b0; dp[0] = d[0] / b0;
                for (int jj = 1; jj < J; jj++) {
                    const double dn = b[jj] - a[jj] * cp[jj - 1];
                    cp[jj] = c[jj] / dn; dp[jj] = (d[jj] - a[jj] * dp[jj - 1]) / dn;
                }
                d[J - 1] = dp[J - 1];
                for (int jj = J - 2; jj >= 0; jj--) d[jj] = dp[jj] - cp[jj] * d[jj + 1];
                if (mm == 0) {
                    double sq = 0.0, sw = 0.0;
                    for (int jj = 0; jj < J; jj++) { const double s_ = fabs(sin(m->the_z[jj + 1])); sq += s_ * d[jj]; sw += s_; }
                    for (int jj = 0; jj < J; jj++) d[jj] -= sq / sw;
                }
            }
        }
        free(a);
    }
    #pragma omp parallel for schedule(static)
    for (int jj = 0; jj < J; jj++) {
        for (int k = 0; k < N; k++) {
            double q = 0.0;
            for (int mm = 0; mm <= NM; mm++) {
                const double w_ = (mm == 0 || 2 * mm == N) ? 1.0 : 2.0;
                q += w_ * (Ac[(size_t)mm * J + jj] * ct[(size_t)mm * N + k]
                         + ((mm == 0 || 2 * mm == N) ? 0.0 : As[(size_t)mm * J + jj] * stb[(size_t)mm * N + k]));
            }
            q /= N;
            for (int i = 0; i < im; i++) X(m, ATSAT_F_P_DYN, i, jj + 1, k) += q;
        }
    }
    free(R); free(ct); free(stb); free(Ac); free(As);
}

/* ---------------- PressureSolver.h:145-766 (pointwise red-black sweeps) ---------------- */
static void pressure(M* m, atsat_dyn_pstats* st) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    double* sinthe_table = (double*)malloc(sizeof(double) * (size_t)jm);
    for (int j = 0; j < jm; j++) {
        sinthe_table[j] = sin(m->the_z[j]);
        if (sinthe_table[j] < p->sinthe_min) sinthe_table[j] = p->sinthe_min;
        if (sinthe_table[j] == 0.0) sinthe_table[j] = 1.0e-5;
    }
    const double p_dyn_cap = p->pdyn_cap;
    const int src_projection = p->press_src;
    const int n_sweeps = p->press_sweeps > 0 ? p->press_sweeps : 1;
    const int press_wall = p->press_wall;
    const int rigid_lid = p->rigid_lid;
    prepare_projection_boundaries(m, rigid_lid);

    const double inv_2dr = 1.0 / (2.0 * m->dr), inv_2dthe = 1.0 / (2.0 * m->dthe), inv_2dphi = 1.0 / (2.0 * m->dphi);
    const double inv_dr2 = 1.0 / (m->dr * m->dr), inv_dthe2 = 1.0 / (m->dthe * m->dthe), inv_dphi2 = 1.0 / (m->dphi * m->dphi);
    const int per = p->phi_periodic;
    const int k_first = per ? 0 : 1;
    const int press_incr = p->press_incr && src_projection != 0;
    const int Su = press_incr ? ATSAT_F_RHS_U : ATSAT_F_AUX_U;
    const int Sv = press_incr ? ATSAT_F_RHS_V : ATSAT_F_AUX_V;
    const int Sw = press_incr ? ATSAT_F_RHS_W : ATSAT_F_AUX_W;
    const size_t n = (size_t)im * jm * km;
    double* lc_old = NULL;
    const int P = ATSAT_F_P_DYN;
    /* the variants of PressureSolver.h:300-308: the radial line pass, and the column-mean correction,
     * which needs the periodic seam and no solid body */
    const int press_line = p->press_line != 0;
    const int press_baro = p->press_baro != 0 && per && !press_wall;
    double* line_rhs = (press_line || press_baro) ? (double*)calloc(n, sizeof(double)) : NULL;

    if (press_incr) {
        lc_old = (double*)calloc(n, sizeof(double));
        #pragma omp parallel for collapse(2) schedule(static)
        for (int i = 1; i < im - 1; i++) {
            for (int j = 1; j < jm - 1; j++) {
                const double rm = metric_radius(m, m->rad_z[i]);
                const double exp_rm = p->coord_stretching ? 1.0 / (rm + 1.0) : 1.0;
                const double num1 = exp_rm * exp_rm * inv_dr2;
                const double num2 = inv_dthe2 / (rm * rm);
                const double num3 = inv_dphi2 / (rm * rm * sinthe_table[j] * sinthe_table[j]);
                for (int k = k_first; k < km - 1; k++) {
                    const int kw = phi_wrap(per, k - 1, km), ke = phi_wrap(per, k + 1, km);
                    const double p0 = X(m, P, i, j, k);
                    double l_;
                    if (press_wall) {
                        l_ = 0.0;
                        l_ += num1 * (X(m, P, i + 1, j, k) - p0);
                        l_ += num1 * (X(m, P, i - 1, j, k) - p0);
                        l_ += num2 * (X(m, P, i, j + 1, k) - p0);
                        l_ += num2 * (X(m, P, i, j - 1, k) - p0);
                        l_ += num3 * (X(m, P, i, j, ke) - p0);
                        l_ += num3 * (X(m, P, i, j, kw) - p0);
                    } else {
                        l_ = num1 * (X(m, P, i + 1, j, k) + X(m, P, i - 1, j, k) - 2.0 * p0)
                           + num2 * (X(m, P, i, j + 1, k) + X(m, P, i, j - 1, k) - 2.0 * p0)
                           + num3 * (X(m, P, i, j, ke) + X(m, P, i, j, kw) - 2.0 * p0);
                    }
                    lc_old[IDX(m, i, j, k)] = l_;
                }
            }
        }
    }

    const double p_mean0 = press_line ? interior_mean(m, k_first) : 0.0;
    double clamped = 0.0, maxupd = 0.0;
    for (int sweep = 0; sweep < n_sweeps; sweep++) {
        double mu = 0.0;
        for (int colour = 0; colour < 2; colour++) {
            #pragma omp parallel for collapse(2) schedule(static) reduction(+:clamped) reduction(max:mu)
            for (int i = 1; i < im - 1; i++) {
                for (int j = 1; j < jm - 1; j++) {
                    Geo g;
                    make_geo(m, i, sinthe_table[j], cos(m->the_z[j]), &g);
                    const double num1 = g.exp_2_rm * inv_dr2;
                    const double num2 = g.inv_rm2 * inv_dthe2;
                    const double num3 = g.inv_rm2sinthe2 * inv_dphi2;
                    const double denom = 2.0 * num1 + 2.0 * num2 + 2.0 * num3;
                    for (int k = k_first; k < km - 1; k++) {
                        if (((i + j + k) & 1) != colour) continue;
                        const int kw = phi_wrap(per, k - 1, km), ke = phi_wrap(per, k + 1, km);
                        double du_dr, dv_dthe, dw_dphi;
                        if (src_projection == 0) {
                            du_dr = ((X(m, ATSAT_F_AUX_U, i + 1, j, k) - X(m, ATSAT_F_AUX_U, i - 1, j, k))
                                   - (X(m, ATSAT_F_RHS_U, i + 1, j, k) - X(m, ATSAT_F_RHS_U, i - 1, j, k))) * inv_2dr;
                            dv_dthe = ((X(m, ATSAT_F_AUX_V, i, j + 1, k) - X(m, ATSAT_F_AUX_V, i, j - 1, k))
                                     - (X(m, ATSAT_F_RHS_V, i, j + 1, k) - X(m, ATSAT_F_RHS_V, i, j - 1, k))) * inv_2dthe;
                            dw_dphi = ((X(m, ATSAT_F_AUX_W, i, j, ke) - X(m, ATSAT_F_AUX_W, i, j, kw))
                                     - (X(m, ATSAT_F_RHS_W, i, j, ke) - X(m, ATSAT_F_RHS_W, i, j, kw))) * inv_2dphi;
                        } else {
                            const double sup = (press_incr && rigid_lid && (i + 1 == im - 1)) ? 0.0 : X(m, Su, i + 1, j, k);
                            const double sum_ = (press_incr && rigid_lid && (i - 1 == 0)) ? 0.0 : X(m, Su, i - 1, j, k);
                            du_dr = (sup - sum_) * inv_2dr;
                            dv_dthe = (X(m, Sv, i, j + 1, k) - X(m, Sv, i, j - 1, k)) * inv_2dthe;
                            dw_dphi = (X(m, Sw, i, j, ke) - X(m, Sw, i, j, kw)) * inv_2dphi;
                        }
                        double div_src = du_dr * g.exp_rm + dv_dthe * g.inv_rm + dw_dphi * g.inv_rmsinthe;
                        double acc = 0.0, den = denom;
                        if (press_wall) {
                            acc = den = 0.0;
                            acc += num1 * X(m, P, i + 1, j, k); den += num1;
                            acc += num1 * X(m, P, i - 1, j, k); den += num1;
                            acc += num2 * X(m, P, i, j + 1, k); den += num2;
                            acc += num2 * X(m, P, i, j - 1, k); den += num2;
                            acc += num3 * X(m, P, i, j, ke); den += num3;
                            acc += num3 * X(m, P, i, j, kw); den += num3;
                            if (den <= 0.0) continue;
                        } else {
                            acc = (X(m, P, i + 1, j, k) + X(m, P, i - 1, j, k)) * num1
                                + (X(m, P, i, j + 1, k) + X(m, P, i, j - 1, k)) * num2
                                + (X(m, P, i, j, ke) + X(m, P, i, j, kw)) * num3;
                        }
                        const double src_max = den * p_dyn_cap;
                        if (!isfinite(div_src)) { div_src = 0.0; clamped += 1.0; }
                        else if (div_src > src_max) { div_src = src_max; clamped += 1.0; }
                        else if (div_src < -src_max) { div_src = -src_max; clamped += 1.0; }
                        if (press_incr) div_src += lc_old[IDX(m, i, j, k)];
                        if (line_rhs) line_rhs[IDX(m, i, j, k)] = div_src;
                        const double old = X(m, P, i, j, k);
                        const double nv = (acc - div_src) / den;
                        X(m, P, i, j, k) = nv;
                        const double dd = fabs(nv - old);
                        if (dd > mu) mu = dd;
                    }
                }
            }
        }
        maxupd = mu;
        if (press_line) line_pass(m, sinthe_table, line_rhs, k_first, inv_dr2, inv_dthe2, inv_dphi2);
        if (press_baro) barotropic_pass(m, sinthe_table, line_rhs, inv_dr2, inv_dthe2, inv_dphi2);
        /* outer boundary of the relaxation, PressureSolver.h:718-746 */
        #pragma omp parallel for collapse(2)
        for (int k = 0; k < km; k++) {
            for (int j = 0; j < jm; j++) {
                X(m, P, 0, j, k) = c43 * X(m, P, 1, j, k) - c13 * X(m, P, 2, j, k);
                X(m, P, im - 1, j, k) = c43 * X(m, P, im - 2, j, k) - c13 * X(m, P, im - 3, j, k);
            }
        }
        #pragma omp parallel for collapse(2)
        for (int k = 0; k < km; k++) {
            for (int i = 0; i < im; i++) {
                X(m, P, i, 0, k) = c43 * X(m, P, i, 1, k) - c13 * X(m, P, i, 2, k);
                X(m, P, i, jm - 1, k) = c43 * X(m, P, i, jm - 2, k) - c13 * X(m, P, i, jm - 3, k);
            }
        }
        #pragma omp parallel for collapse(2)
        for (int i = 0; i < im; i++) {
            for (int j = 0; j < jm; j++) {
                if (per) { X(m, P, i, j, km - 1) = X(m, P, i, j, 0); continue; }
                X(m, P, i, j, 0) = c43 * X(m, P, i, j, 1) - c13 * X(m, P, i, j, 2);
                X(m, P, i, j, km - 1) = c43 * X(m, P, i, j, km - 2) - c13 * X(m, P, i, j, km - 3);
                X(m, P, i, j, 0) = X(m, P, i, j, km - 1) = (X(m, P, i, j, 0) + X(m, P, i, j, km - 1)) / 2.0;
            }
        }
        /* PRESS_LINE holds the all-Neumann constant: one shift of every cell (PressureSolver.h:750-755) */
        if (press_line) {
            const double shift = interior_mean(m, k_first) - p_mean0;
            double* pd = m->f[P];
            for (size_t c = 0; c < n; c++) pd[c] -= shift;
        }
    }
    if (st) { st->sweeps = n_sweeps; st->src_clamped = clamped; st->max_abs_update = maxupd; }
    free(line_rhs);
    free(lc_old);
    free(sinthe_table);
}

/* ---------------- AtomUtils::damp_wiggles, lib/Utils.cpp:229-322 (no surface mask) ----------------
 * The 1-2-1 filter f += strength/4 (f[-1] - 2 f + f[+1]) along k (periodic over the km-1 distinct
 * meridians with k = km-1 their copy when the seam is periodic, else over all km), then j (clamped at
 * the poles), then i (clamped at the walls); each pass reads a copy of the field. */
static void damp_wiggles(M* m, int fid, int along_i, int along_j, int along_k, double strength, int passes) {
    const int im = m->im, jm = m->jm, km = m->km;
    const size_t n = (size_t)im * jm * km;
    const double coeff = strength * 0.25;
    double* f = m->f[fid];
    double* tmp = (double*)malloc(n * sizeof(double));
    for (int pass = 0; pass < passes; ++pass) {
        if (along_k) {
            memcpy(tmp, f, n * sizeof(double));
            const int seam = m->p->phi_periodic && km > 2;
            const int k_end = seam ? km - 1 : km;
            #pragma omp parallel for collapse(2) schedule(static)
            for (int i = 0; i < im; ++i)
                for (int j = 0; j < jm; ++j) {
                    for (int k = 0; k < k_end; ++k) {
                        const int km1 = seam ? (k == 0 ? km - 2 : k - 1) : (k - 1 + km) % km;
                        const int kp1 = seam ? (k == km - 2 ? 0 : k + 1) : (k + 1) % km;
                        const double t0 = tmp[IDX(m, i, j, k)];
                        f[IDX(m, i, j, k)] = t0 + coeff * (tmp[IDX(m, i, j, km1)] - 2.0 * t0 + tmp[IDX(m, i, j, kp1)]);
                    }
                    if (seam) f[IDX(m, i, j, km - 1)] = f[IDX(m, i, j, 0)];
                }
        }
        if (along_j) {
            memcpy(tmp, f, n * sizeof(double));
            #pragma omp parallel for collapse(2) schedule(static)
            for (int i = 0; i < im; ++i)
                for (int j = 0; j < jm; ++j) {
                    const int jm1 = j - 1 < 0 ? 0 : j - 1, jp1 = j + 1 > jm - 1 ? jm - 1 : j + 1;
                    for (int k = 0; k < km; ++k) {
                        const double t0 = tmp[IDX(m, i, j, k)];
                        f[IDX(m, i, j, k)] = t0 + coeff * (tmp[IDX(m, i, jm1, k)] - 2.0 * t0 + tmp[IDX(m, i, jp1, k)]);
                    }
                }
        }
        if (along_i) {
            memcpy(tmp, f, n * sizeof(double));
            #pragma omp parallel for collapse(2) schedule(static)
            for (int j = 0; j < jm; ++j)
                for (int k = 0; k < km; ++k)
                    for (int i = 0; i < im; ++i) {
                        const int im1 = i - 1 < 0 ? 0 : i - 1, ip1 = i + 1 > im - 1 ? im - 1 : i + 1;
                        const double t0 = tmp[IDX(m, i, j, k)];
                        f[IDX(m, i, j, k)] = t0 + coeff * (tmp[IDX(m, im1, j, k)] - 2.0 * t0 + tmp[IDX(m, ip1, j, k)]);
                    }
        }
    }
    free(tmp);
}

/* the p_dyn filter of cSaturnModel::Run after the pressure call (cSaturnModel.cpp:894-897) */
static void damp_pdyn(M* m) {
    const int mode = m->p->damp_pdyn;
    if (mode == 1) damp_wiggles(m, ATSAT_F_P_DYN, 1, 1, 1, 1.0, 1);
    else if (mode == 2) damp_wiggles(m, ATSAT_F_P_DYN, 1, 0, 0, 1.0, 1);
    else if (mode == 3) damp_wiggles(m, ATSAT_F_P_DYN, 1, 0, 1, 1.0, 1);
}

/* ---------------- cSaturnModel::clampNegativeSpecies, FileIO_Sat.cpp:716-772 ----------------
 * budget (optional): 4 x 11 doubles, the finite amount clipped, the cells, and both again for the radial
 * planes i = 0, im-1, per species in the reference's order, added to what they hold. */
static const int CLAMP_SPECIES[11] = { ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                                       ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                                       ATSAT_F_CH4_ICE, ATSAT_F_NH4SH };

static void clamp_negative_species(M* m, double* budget) {
    if (!m->p->clamp_species) return;
    const int im = m->im, jm = m->jm, km = m->km;
    for (int q = 0; q < 11; q++) {
        double* F = m->f[CLAMP_SPECIES[q]];
        double added = 0.0, added_bnd = 0.0;
        long cells = 0, cells_bnd = 0;
        #pragma omp parallel for collapse(2) schedule(static) reduction(+:added, cells, added_bnd, cells_bnd)
        for (int i = 0; i < im; i++)
            for (int j = 0; j < jm; j++)
                for (int k = 0; k < km; k++) {
                    const double v = F[IDX(m, i, j, k)];
                    if (!(v >= 0.0)) {
                        if (isfinite(v)) {
                            added -= v; cells++;
                            if (i == 0 || i == im - 1) { added_bnd -= v; cells_bnd++; }
                        }
                        F[IDX(m, i, j, k)] = 0.0;
                    }
                }
        if (budget) {
            budget[q] += added;
            budget[11 + q] += (double)cells;
            budget[22 + q] += added_bnd;
            budget[33 + q] += (double)cells_bnd;
        }
    }
}

/* ---------------- Turbulence<cSaturnModel>::run, planet/Turbulence.h:306-329 ----------------
 * ATSAT has no solid body (cSaturnModel.h:254-255: surface_index 0, is_solid false), so the land branches
 * are constant. Layer heights are the model's float table (cSaturnModel.h:1062-1074): h = (float)(L_atm dr),
 * height(i) = (float)i * h km. cp for the lapse rate is cp_mix (CpH2.h:129-131, ATSAT keeps it in the
 * dynamics). prod is the closure's production array (im*jm*km), vel_star its u_tau (jm*km). */
typedef struct {
    const M* m;
    const atsat_dyn_turb_params* tp;
    float h;                     /* the layer spacing in km, as the model's float table holds it */
    double L_m, nue_air, re_turb;
} TurbCtx;

static inline double t_height_m(const TurbCtx* c, int i) {
    if (0 > i || i > c->m->im - 1) return (double)(-1.0f) * 1.0e3;
    return (double)((float)i * c->h) * 1.0e3;
}
static inline double t_layer_thickness_m(const TurbCtx* c, int i) {
    if (i < 0 || i > c->m->im - 2) return 0.0;
    return (double)((float)(i + 1) * c->h - (float)i * c->h) * 1.0e3;
}
static inline double clamp3(double x, double lo, double hi) { return (x < lo) ? lo : ((x > hi) ? hi : x); }

#define TK(i, j, k) X(m, ATSAT_F_TKE, i, j, k)
#define DS(i, j, k) X(m, ATSAT_F_DIS, i, j, k)

static void turb_sst(const TurbCtx* c, double* prod, int i, int j, int k, double y_mount, double rm, double sinthe,
                     double dtkedr, double ddisdr, double Omega) {
    M* m = (M*)c->m;
    const double a1 = 0.31, bet_star = 0.09, bet1 = 0.0333, bet2 = 0.0368, gam1 = 0.413, gam2 = 0.2, sig_w2 = 1.168;
    const double L_m = c->L_m;
    const double nue_air_nd = c->nue_air / (m->p->u_0 * L_m);
    const double dz_layer = smax(1.0, t_layer_thickness_m(c, (i - 1 > 0) ? i - 1 : 0));
    const double y_phys = c->tp->turb_free ? 1.0e20 : smax(t_height_m(c, i) - y_mount, dz_layer);
    const double y_star = y_phys / L_m;
    const double rmsinthe = rm * sinthe;
    const int per = m->p->phi_periodic;
    const int kw = phi_wrap(per, k - 1, m->km), ke = phi_wrap(per, k + 1, m->km);
    const double dtkedthe = (TK(i, j + 1, k) - TK(i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double ddisdthe = (DS(i, j + 1, k) - DS(i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double dtkedphi = (TK(i, j, ke) - TK(i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double ddisdphi = (DS(i, j, ke) - DS(i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double grad_dot = dtkedr * ddisdr + dtkedthe * ddisdthe + dtkedphi * ddisdphi;
    const double CD_kw = smax(2.0 * sig_w2 / smax(DS(i, j, k), 1.0e-20) * grad_dot, 1.0e-20);
    const double dis_safe = smax(DS(i, j, k), 1.0e-20);
    const double arg1 = smin(smax(sqrt(TK(i, j, k)) / (bet_star * dis_safe * y_star),
                                  500.0 * nue_air_nd / (y_star * y_star * dis_safe)),
                             4.0 * sig_w2 * TK(i, j, k) / (CD_kw * y_star * y_star));
    const double arg2 = smax(2.0 * sqrt(TK(i, j, k)) / (bet_star * dis_safe * y_star),
                             500.0 * nue_air_nd / (y_star * y_star * dis_safe));
    const double F1 = tanh(pow(arg1, 4));
    const double F2 = tanh(pow(arg2, 2));
    X(m, ATSAT_F_NUE, i, j, k) = a1 * TK(i, j, k) / smax(a1 * dis_safe, Omega * F2);
    const double tke_safe = smax(TK(i, j, k), 1.0e-20);
    const double P_k = smin(prod[IDX(m, i, j, k)], 20.0 * bet_star * tke_safe * dis_safe);
    const double Y_k = bet_star * tke_safe * dis_safe;
    const double P_w = (F1 * gam1 + (1.0 - F1) * gam2) * P_k * dis_safe / tke_safe;
    const double Y_w = (F1 * bet1 + (1.0 - F1) * bet2) * dis_safe * dis_safe;
    const double D_w = 2.0 * (1.0 - F1) * sig_w2 / dis_safe * grad_dot;
    X(m, ATSAT_F_TKE_SOURCE, i, j, k) = P_k - Y_k;
    X(m, ATSAT_F_DIS_SOURCE, i, j, k) = P_w - Y_w + D_w;
}

static void turb_k_omega(const TurbCtx* c, double* prod, int i, int j, int k, double dtkedr, double ddisdr,
                         double Omega_mag) {
    M* m = (M*)c->m;
    const double bet_star = 0.09, gam = 0.52, C_lim = 0.875, bet_0 = 0.0708;
    const double rm = metric_radius(m, m->rad_z[i]);
    double sinthe = sin(m->the_z[j]);
    if (sinthe == 0.0) sinthe = 1.0e-5;
    const double rmsinthe = rm * sinthe;
    const int per = m->p->phi_periodic;
    const int kw = phi_wrap(per, k - 1, m->km), ke = phi_wrap(per, k + 1, m->km);
    const double dtkedthe_neu = (TK(i, j + 1, k) - TK(i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double ddisdthe_neu = (DS(i, j + 1, k) - DS(i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double dtkedphi_neu = (TK(i, j, ke) - TK(i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double ddisdphi_neu = (DS(i, j, ke) - DS(i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double dudr = (X(m, ATSAT_F_U, i + 1, j, k) - X(m, ATSAT_F_U, i - 1, j, k)) / (2.0 * m->dr) / (rm + 1.0);
    const double dvdthe = (X(m, ATSAT_F_V, i, j + 1, k) - X(m, ATSAT_F_V, i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double dwdphi = (X(m, ATSAT_F_W, i, j, ke) - X(m, ATSAT_F_W, i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double dudthe_u = (X(m, ATSAT_F_U, i, j + 1, k) - X(m, ATSAT_F_U, i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double dudphi_u = (X(m, ATSAT_F_U, i, j, ke) - X(m, ATSAT_F_U, i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double dvdr_u = (X(m, ATSAT_F_V, i + 1, j, k) - X(m, ATSAT_F_V, i - 1, j, k)) / (2.0 * m->dr) / (rm + 1.0);
    const double dwdr_u = (X(m, ATSAT_F_W, i + 1, j, k) - X(m, ATSAT_F_W, i - 1, j, k)) / (2.0 * m->dr) / (rm + 1.0);
    const double dvdphi_u = (X(m, ATSAT_F_V, i, j, ke) - X(m, ATSAT_F_V, i, j, kw)) / (rmsinthe * 2.0 * m->dphi);
    const double dwdthe_u = (X(m, ATSAT_F_W, i, j + 1, k) - X(m, ATSAT_F_W, i, j - 1, k)) / (rm * 2.0 * m->dthe);
    const double S11 = dudr, S22 = dvdthe, S33 = dwdphi;
    const double S12 = 0.5 * (dudthe_u + dvdr_u);
    const double S13 = 0.5 * (dudphi_u + dwdr_u);
    const double S23 = 0.5 * (dvdphi_u + dwdthe_u);
    const double S_mag = sqrt(2.0 * (S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23)));
    const double w_hat = smax(DS(i, j, k), C_lim * S_mag / sqrt(bet_star));
    const double gd = dtkedr * ddisdr + dtkedthe_neu * ddisdthe_neu + dtkedphi_neu * ddisdphi_neu;
    const double sig_d = (gd <= 0.0) ? 0.0 : 0.125;
    const double chi_w = fabs(Omega_mag * Omega_mag * S_mag / pow(bet_star * smax(DS(i, j, k), 1.0e-20), 3));
    const double f_bet = (1.0 + 85.0 * chi_w) / (1.0 + 100.0 * chi_w);
    const double bet_wc = bet_0 * f_bet;
    X(m, ATSAT_F_NUE, i, j, k) = TK(i, j, k) / smax(w_hat, 1.0e-20);
    const double P_k = smin(prod[IDX(m, i, j, k)], 20.0 * bet_star * TK(i, j, k) * DS(i, j, k));
    const double Y_k = bet_star * TK(i, j, k) * DS(i, j, k);
    const double P_w = gam * DS(i, j, k) / smax(TK(i, j, k), 1.0e-20) * P_k;
    const double Y_w = bet_wc * DS(i, j, k) * DS(i, j, k);
    const double D_w = sig_d / smax(DS(i, j, k), 1.0e-20)
                     * (dtkedr * ddisdr + dtkedthe_neu * ddisdthe_neu + dtkedphi_neu * ddisdphi_neu);
    X(m, ATSAT_F_TKE_SOURCE, i, j, k) = P_k - Y_k;
    X(m, ATSAT_F_DIS_SOURCE, i, j, k) = P_w - Y_w + D_w;
}

static void turb_k_epsilon(const TurbCtx* c, double* prod, const double* vel_star, int i, int j, int k, double y_mount) {
    M* m = (M*)c->m;
    const double C_eps_1 = 1.35, C_eps_2 = 1.80, C_nue = 0.028, dis_min = 1.0e-10;
    const double L_m = c->L_m;
    const double y_phys = c->tp->turb_free ? 1.0e20 : smax(t_height_m(c, i) - y_mount, L_m);
    const double y_star = y_phys / L_m;
    X(m, ATSAT_F_NUE, i, j, k) = C_nue * TK(i, j, k) * TK(i, j, k) / smax(DS(i, j, k), dis_min);
    const double d_plus = y_phys * vel_star[(size_t)j * m->km + k] / c->nue_air;
    const double f_nue = 1.0 - exp(-0.0115 * d_plus);
    const double Re_T = TK(i, j, k) * TK(i, j, k) * m->p->u_0 * L_m / smax(DS(i, j, k) * c->nue_air, dis_min * c->nue_air);
    const double f_2 = 1.0 - 0.4 / 1.8 * exp(-Re_T * Re_T / 36.0);
    X(m, ATSAT_F_NUE, i, j, k) *= f_nue;
    const double y_star2 = y_star * y_star;
    const double L_k = -2.0 * TK(i, j, k) / y_star2;
    const double L_w = -2.0 * DS(i, j, k) / y_star2 * exp(-d_plus / 2.0);
    const double P_k = prod[IDX(m, i, j, k)];
    const double Y_k = DS(i, j, k);
    const double tke_safe = smax(TK(i, j, k), dis_min);
    const double P_w = C_eps_1 * DS(i, j, k) / tke_safe * P_k;
    const double Y_w = C_eps_2 * f_2 * DS(i, j, k) * DS(i, j, k) / tke_safe;
    X(m, ATSAT_F_TKE_SOURCE, i, j, k) = P_k - Y_k + L_k / c->re_turb;
    X(m, ATSAT_F_DIS_SOURCE, i, j, k) = P_w - Y_w + L_w / c->re_turb;
}

static void turbulence_run(M* m, const atsat_dyn_turb_params* tp, double* prod, double* vel_star) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const double C_nue = 0.028, Karman = 0.42, dis_min = 1.0e-10;
    (void)Karman;
    TurbCtx c;
    c.m = m;
    c.tp = tp;
    c.h = (float)(p->L_atm * m->dr);
    c.L_m = p->L_atm * 1.0e3;
    c.nue_air = tp->nue_gas;
    c.re_turb = tp->vel_star_ref * tp->z_0 / tp->nue_gas;
    const double u_0 = p->u_0;
    const int per = p->phi_periodic;
    const int k_first = per ? 0 : 1;
    const double nue_max = tp->nue_max_phys / (u_0 * c.L_m);

    /* compute_vel_star (Turbulence.h:335-378) */
    for (int j = 0; j < jm; j++)
        for (int k = 0; k < km; k++) {
            double vs;
            if (tp->turb_free) vs = 0.05;
            else {
                const int i_surf = (0 + 1 < im - 1) ? 0 + 1 : im - 1;
                const double v_s = X(m, ATSAT_F_V, i_surf, j, k), w_s = X(m, ATSAT_F_W, i_surf, j, k);
                const double vw2 = v_s * v_s + w_s * w_s;
                vs = !isfinite(vw2) ? 0.05 : clamp3(sqrt(0.002) * (u_0 * sqrt(vw2)), 0.05, tp->vel_star_max);
            }
            vel_star[(size_t)j * km + k] = vs;
        }

    /* compute_sources (Turbulence.h:613-882) */
    const double k_bg_free = tp->k_bg / (u_0 * u_0);
    #define K_BG_OF(j, k) (tp->turb_free ? k_bg_free \
        : 0.01 * vel_star[(size_t)(j) * km + (k)] * vel_star[(size_t)(j) * km + (k)] / (sqrt(C_nue) * u_0 * u_0))
    if (tp->clamp_pass) {
        for (int j = 1; j < jm - 1; j++)
            for (int k = k_first; k < km - 1; k++)
                for (int i = 1; i < im - 1; i++) {
                    TK(i, j, k) = smax(0.0, TK(i, j, k));
                    DS(i, j, k) = smax(dis_min, DS(i, j, k));
                }
    }
    #pragma omp parallel for collapse(2) schedule(static)
    for (int j = 1; j < jm - 1; j++) {
        for (int k = k_first; k < km - 1; k++) {
            const int kw = phi_wrap(per, k - 1, km), ke = phi_wrap(per, k + 1, km);
            const double y_mount = t_height_m(&c, 0);
            const double k_bg_nd = K_BG_OF(j, k);
            for (int i = 1; i < im - 1; i++) {
                const double rm = metric_radius(m, m->rad_z[i]);
                const double exp_rm = p->coord_stretching ? 1.0 / (rm + 1.0) : 1.0;
                double sinthe = sin(m->the_z[j]);
                if (sinthe == 0.0) sinthe = 1.0e-5;
                const double costhe = cos(m->the_z[j]);
                const double cotanthe = costhe / sinthe;
                const double inv_rm = 1.0 / rm;
                const double rmsinthe = rm * sinthe;
                const double inv_2dr = 1.0 / (2.0 * m->dr);
                const double inv_2dthe = 1.0 / (2.0 * m->dthe);
                const double inv_2dphi = 1.0 / (2.0 * m->dphi);
                const double inv_rm2dthe = inv_2dthe / rm;
                const double inv_rmsinthe2dphi = inv_2dphi / rmsinthe;
                if (!tp->clamp_pass) { TK(i, j, k) = smax(0.0, TK(i, j, k)); DS(i, j, k) = smax(dis_min, DS(i, j, k)); }
                const double dudr = (X(m, ATSAT_F_U, i + 1, j, k) - X(m, ATSAT_F_U, i - 1, j, k)) * inv_2dr * exp_rm;
                const double dvdr = (X(m, ATSAT_F_V, i + 1, j, k) - X(m, ATSAT_F_V, i - 1, j, k)) * inv_2dr * exp_rm;
                const double dwdr = (X(m, ATSAT_F_W, i + 1, j, k) - X(m, ATSAT_F_W, i - 1, j, k)) * inv_2dr * exp_rm;
                const double dudthe = (X(m, ATSAT_F_U, i, j + 1, k) - X(m, ATSAT_F_U, i, j - 1, k)) * inv_rm2dthe;
                const double dvdthe = (X(m, ATSAT_F_V, i, j + 1, k) - X(m, ATSAT_F_V, i, j - 1, k)) * inv_rm2dthe;
                const double dwdthe = (X(m, ATSAT_F_W, i, j + 1, k) - X(m, ATSAT_F_W, i, j - 1, k)) * inv_rm2dthe;
                const double dudphi = (X(m, ATSAT_F_U, i, j, ke) - X(m, ATSAT_F_U, i, j, kw)) * inv_rmsinthe2dphi;
                const double dvdphi = (X(m, ATSAT_F_V, i, j, ke) - X(m, ATSAT_F_V, i, j, kw)) * inv_rmsinthe2dphi;
                const double dwdphi = (X(m, ATSAT_F_W, i, j, ke) - X(m, ATSAT_F_W, i, j, kw)) * inv_rmsinthe2dphi;
                const double dtkedr = (TK(i + 1, j, k) - TK(i - 1, j, k)) * inv_2dr * exp_rm;
                const double ddisdr = (DS(i + 1, j, k) - DS(i - 1, j, k)) * inv_2dr * exp_rm;
                double cnue;
                {
                    const double dis_here = smax(DS(i, j, k), dis_min);
                    const double tke_here = smax(TK(i, j, k), 0.0);
                    cnue = (tp->model == ATSAT_TURB_K_EPSILON) ? C_nue * tke_here * tke_here / dis_here
                                                               : tke_here / dis_here;
                    cnue = smin(cnue, nue_max);
                }
                const double u_r = tp->curv ? X(m, ATSAT_F_U, i, j, k) * inv_rm : 0.0;
                const double v_r = tp->curv ? X(m, ATSAT_F_V, i, j, k) * inv_rm : 0.0;
                const double w_r = tp->curv ? X(m, ATSAT_F_W, i, j, k) * inv_rm : 0.0;
                const double v_cot_r = v_r * cotanthe;
                const double w_cot_r = w_r * cotanthe;
                const double g_rr = dudr, g_rt = dudthe - v_r, g_rp = dudphi - w_r;
                const double g_tr = dvdr, g_tt = dvdthe + u_r, g_tp = dvdphi - w_cot_r;
                const double g_pr = dwdr, g_pt = dwdthe, g_pp = dwdphi + u_r + v_cot_r;
                const double der = 0.66667 * (g_rr + g_tt + g_pp);
                const double tk = TK(i, j, k);
                prod[IDX(m, i, j, k)] = smax(0.0,
                      (cnue * (2.0 * g_rr - der) - 0.66667 * tk) * g_rr
                    + (cnue * (g_rt + g_tr))                     * g_rt
                    + (cnue * (g_rp + g_pr))                     * g_rp
                    + (cnue * (2.0 * g_tt - der) - 0.66667 * tk) * g_tt
                    + (cnue * (g_tr + g_rt))                     * g_tr
                    + (cnue * (g_tp + g_pt))                     * g_tp
                    + (cnue * (2.0 * g_pp - der) - 0.66667 * tk) * g_pp
                    + (cnue * (g_pr + g_rp))                     * g_pr
                    + (cnue * (g_pt + g_tp))                     * g_pt);
                const double W12 = g_rt - g_tr, W13 = g_rp - g_pr, W23 = g_tp - g_pt;
                const double Omega = sqrt(W12 * W12 + W13 * W13 + W23 * W23);
                if (tp->model == ATSAT_TURB_K_EPSILON) turb_k_epsilon(&c, prod, vel_star, i, j, k, y_mount);
                else if (tp->model == ATSAT_TURB_K_OMEGA) turb_k_omega(&c, prod, i, j, k, dtkedr, ddisdr, Omega);
                else turb_sst(&c, prod, i, j, k, y_mount, rm, sinthe, dtkedr, ddisdr, Omega);
                if (tp->buoy != 0) {
                    const double Pr_t = 0.9;
                    const double T = X(m, ATSAT_F_T, i, j, k) * p->t_ref;
                    const double dz = t_height_m(&c, i + 1) - t_height_m(&c, i - 1);
                    const double dTdz = (X(m, ATSAT_F_T, i + 1, j, k) - X(m, ATSAT_F_T, i - 1, j, k)) * p->t_ref / dz;
                    const double cp = p->cp_mix;
                    double Gam = p->g / cp, fac = 1.0;
                    if (tp->buoy == 3 && T > 0.0) {
                        double rho = p->r_mix;
                        if (p->local_rho) {
                            const double r_ = X(m, ATSAT_F_RHO_MIX, i, j, k);
                            rho = (r_ > 0.0 && isfinite(r_)) ? r_ : p->r_mix;
                        }
                        double A = 0.0, B = 0.0;
                        static const int gv_[3] = { ATSAT_F_H2O, ATSAT_F_NH3, ATSAT_F_CH4 };
                        static const int gc_[3] = { ATSAT_F_H2O_CLOUD, ATSAT_F_NH3_CLOUD, ATSAT_F_CH4_CLOUD };
                        static const int gi_[3] = { ATSAT_F_H2O_ICE, ATSAT_F_NH3_ICE, ATSAT_F_CH4_ICE };
                        for (int n = 0; rho > 0.0 && n < 3; n++) {
                            const double qc = (smax(0.0, X(m, gc_[n], i, j, k)) + smax(0.0, X(m, gi_[n], i, j, k))) / rho;
                            if (!(qc > 1.0e-9)) continue;
                            const double qv = smax(0.0, X(m, gv_[n], i, j, k)) / rho;
                            const double L = T >= tp->t_0[n] ? tp->lv[n] : tp->ls[n];
                            A += L * qv / (p->R_mix * T);
                            B += tp->ep[n] * L * L * qv / (cp * p->R_mix * T * T);
                        }
                        if (isfinite(A + B)) { Gam *= (1.0 + A) / (1.0 + B); fac = 1.0 + A; }
                    }
                    const double N2 = (T > 0.0 && dz > 0.0) ? p->g / T * (dTdz + Gam) * fac : 0.0;
                    if (isfinite(N2) && (N2 > 0.0 || tp->buoy == 2)) {
                        const double tL = c.L_m / u_0;
                        X(m, ATSAT_F_TKE_SOURCE, i, j, k) -= smax(0.0, X(m, ATSAT_F_NUE, i, j, k)) * N2 * tL * tL / Pr_t;
                    }
                }
                if (!tp->clamp_pass) {
                    TK(i, j, k) = smax(k_bg_nd, TK(i, j, k));
                    DS(i, j, k) = smax(dis_min, DS(i, j, k));
                    X(m, ATSAT_F_NUE, i, j, k) = clamp3(X(m, ATSAT_F_NUE, i, j, k), 0.0, nue_max);
                    const double dsm = 20.0 * DS(i, j, k) * DS(i, j, k);
                    X(m, ATSAT_F_DIS_SOURCE, i, j, k) = clamp3(X(m, ATSAT_F_DIS_SOURCE, i, j, k), -dsm, dsm);
                    const double tsm = 20.0 * TK(i, j, k) * DS(i, j, k);
                    X(m, ATSAT_F_TKE_SOURCE, i, j, k) = clamp3(X(m, ATSAT_F_TKE_SOURCE, i, j, k), -tsm, tsm);
                }
            }
        }
    }
    if (tp->clamp_pass) {
        for (int j = 1; j < jm - 1; j++)
            for (int k = k_first; k < km - 1; k++) {
                const double k_bg_nd = K_BG_OF(j, k);
                for (int i = 1; i < im - 1; i++) {
                    TK(i, j, k) = smax(k_bg_nd, TK(i, j, k));
                    DS(i, j, k) = smax(dis_min, DS(i, j, k));
                    X(m, ATSAT_F_NUE, i, j, k) = clamp3(X(m, ATSAT_F_NUE, i, j, k), 0.0, nue_max);
                    const double dsm = 20.0 * DS(i, j, k) * DS(i, j, k);
                    X(m, ATSAT_F_DIS_SOURCE, i, j, k) = clamp3(X(m, ATSAT_F_DIS_SOURCE, i, j, k), -dsm, dsm);
                    const double tsm = 20.0 * TK(i, j, k) * DS(i, j, k);
                    X(m, ATSAT_F_TKE_SOURCE, i, j, k) = clamp3(X(m, ATSAT_F_TKE_SOURCE, i, j, k), -tsm, tsm);
                }
            }
    }
    #undef K_BG_OF

    /* apply_wall_bc (Turbulence.h:382-423): no obstacle, so the zero-gradient copy at i = 0 everywhere */
    for (int j = 0; j < jm; j++)
        for (int k = 0; k < km; k++) {
            TK(0, j, k) = TK(1, j, k);
            DS(0, j, k) = DS(1, j, k);
            X(m, ATSAT_F_NUE, 0, j, k) = X(m, ATSAT_F_NUE, 1, j, k);
        }

    /* clamp_nue (Turbulence.h:564-589) */
    {
        int i_abl = 0;
        while (i_abl < im - 1 && t_height_m(&c, i_abl) <= tp->abl_height) i_abl++;
        const double taper_dz = smax(1.0, t_height_m(&c, i_abl < im - 1 ? i_abl : im - 1)
                                        - t_height_m(&c, i_abl - 1 > 0 ? i_abl - 1 : 0));
        for (int i = 0; i < im; i++)
            for (int j = 0; j < jm; j++)
                for (int k = 0; k < km; k++) {
                    double f = 1.0;
                    if (tp->abl_taper) {
                        const double z_agl = t_height_m(&c, i) - t_height_m(&c, 0);
                        f = clamp3((tp->abl_height + taper_dz - z_agl) / taper_dz, 0.0, 1.0);
                    }
                    X(m, ATSAT_F_NUE, i, j, k) = clamp3(X(m, ATSAT_F_NUE, i, j, k), 0.0, nue_max) * f;
                }
    }

    /* seam_copy (Turbulence.h:542-561) */
    if (per) {
        const int fl[7] = { ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_TKEN, ATSAT_F_DISN, ATSAT_F_NUE,
                            ATSAT_F_TKE_SOURCE, ATSAT_F_DIS_SOURCE };
        for (int i = 0; i < im; i++)
            for (int j = 0; j < jm; j++) {
                for (int q = 0; q < 7; q++) X(m, fl[q], i, j, km - 1) = X(m, fl[q], i, j, 0);
                prod[IDX(m, i, j, km - 1)] = prod[IDX(m, i, j, 0)];
            }
    }

    /* fill_lid_corners (Turbulence.h:510-540); ATSAT treats the closure's arrays in its own boundary
     * conditions (bc_turb_active = turb_active), so only the two lid corners get the mean */
    if (tp->turb_free) {
        const int il = im - 1;
        if (!p->turb_active) {
            /* bc_turb_active false: the whole lid and both pole rows by the zero-gradient copy */
            const int fl[7] = { ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_TKEN, ATSAT_F_DISN, ATSAT_F_NUE,
                                ATSAT_F_TKE_SOURCE, ATSAT_F_DIS_SOURCE };
            for (int j = 1; j < jm - 1; j++)
                for (int k = 0; k < km; k++) {
                    for (int q = 0; q < 7; q++) X(m, fl[q], il, j, k) = X(m, fl[q], il - 1, j, k);
                    prod[IDX(m, il, j, k)] = prod[IDX(m, il - 1, j, k)];
                }
            for (int i = 0; i < im; i++)
                for (int k = 0; k < km; k++) {
                    for (int q = 0; q < 7; q++) {
                        X(m, fl[q], i, 0, k) = X(m, fl[q], i, 1, k);
                        X(m, fl[q], i, jm - 1, k) = X(m, fl[q], i, jm - 2, k);
                    }
                    prod[IDX(m, i, 0, k)] = prod[IDX(m, i, 1, k)];
                    prod[IDX(m, i, jm - 1, k)] = prod[IDX(m, i, jm - 2, k)];
                }
        } else {
            /* the reference's array order: tke, dis, tken, disn, nue, prod, tke_source, dis_source */
            for (int k = 0; k < km; k++) {
                for (int q = 0; q < 8; q++) {
                    double* a = (q == 5) ? prod : m->f[q < 5 ? (int[]){ ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_TKEN,
                                                                        ATSAT_F_DISN, ATSAT_F_NUE }[q]
                                                             : (q == 6 ? ATSAT_F_TKE_SOURCE : ATSAT_F_DIS_SOURCE)];
                    a[IDX(m, il, 0, k)] = 0.5 * (a[IDX(m, il, 1, k)] + a[IDX(m, il - 1, 0, k)]);
                    a[IDX(m, il, jm - 1, k)] = 0.5 * (a[IDX(m, il, jm - 2, k)] + a[IDX(m, il - 1, jm - 1, k)]);
                }
            }
        }
    }
}
#undef TK
#undef DS

/* ---------------- cSaturnModel.cpp:1551-1600 ---------------- */
static void restore_var(M* m) {
    const size_t n = (size_t)m->im * m->jm * m->km;
    for (int q = 0; q < ATSAT_NPROG; q++) memcpy(m->f[ATSAT_F_N_BASE + q], m->f[q], n * sizeof(double));
    memcpy(m->f[ATSAT_F_P_DYNN], m->f[ATSAT_F_P_DYN], n * sizeof(double));
}

/* ---------------- BoundaryConditions.h:150-518 with BC_Sat.cpp:61-179 ----------------
 * bcTheta, bcPhi, bcRadius (and BC_Sat's species lid/wall copies) in the order cSaturnModel::Run
 * calls them (cSaturnModel.cpp:1091-1093), restricted to the fields of the dycore. */
static inline double bc_form(int form, double a, double b, double c) {
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int f = (form == 0) ? 3 : form;          /* ATSAT's bc_default_form() is CUBIC */
    if (f == 1) return a;
    if (f == 2) return c43 * a - c13 * b;
    return c - 3.0 * b + 3.0 * a;
}

static const int BC_RADIUS[] = { ATSAT_F_T, ATSAT_F_U, ATSAT_F_V, ATSAT_F_W, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
    ATSAT_F_CH4_ICE, ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3, ATSAT_F_NH3_CLOUD,
    ATSAT_F_NH3_ICE, ATSAT_F_NH4SH, ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH,
    ATSAT_F_FLUXLIM_NH4SH, ATSAT_F_THERMALMASSFLUX };
static const int BC_THETA_EXTRAP[] = { ATSAT_F_T, ATSAT_F_U, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD, ATSAT_F_CH4_ICE,
    ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3, ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE,
    ATSAT_F_NH4SH, ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH, ATSAT_F_THERMALMASSFLUX };
static const int BC_THETA_ZERO[] = { ATSAT_F_V, ATSAT_F_W, ATSAT_F_FLUXLIM_NH4SH };
static const int BC_TURB[] = { ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_NUE };
static const double BC_TURB_FLOOR[] = { 0.0, 1.0e-10, 0.0 };
static const int BC_SPECIES[] = { ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
    ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD, ATSAT_F_CH4_ICE, ATSAT_F_NH4SH };
#define NELEM(a) ((int)(sizeof(a) / sizeof((a)[0])))

static void bc_theta(M* m) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int form = p->bc_pole_form;
    const int nfill = p->bc_pole_fill ? 1 : 0;
    const int turb = p->turb_active;
    const int k_lo = p->phi_periodic ? 0 : 1;
    #pragma omp parallel for
    for (int k = k_lo; k < km - 1; k++) {
        for (int i = 1; i < im - 1; i++) {
            if (nfill > 0) {
                const int jf = nfill + 1;
                for (int r = 1; r <= nfill; r++) {
                    const double ramp = (double)r / (double)jf;
                    for (int q = 0; q < NELEM(BC_THETA_EXTRAP); q++) {
                        const int F_ = BC_THETA_EXTRAP[q];
                        X(m, F_, i, r, k) = X(m, F_, i, jf, k);
                        X(m, F_, i, jm - 1 - r, k) = X(m, F_, i, jm - 1 - jf, k);
                    }
                    for (int q = 0; q < NELEM(BC_THETA_ZERO); q++) {
                        const int F_ = BC_THETA_ZERO[q];
                        X(m, F_, i, r, k) = ramp * X(m, F_, i, jf, k);
                        X(m, F_, i, jm - 1 - r, k) = ramp * X(m, F_, i, jm - 1 - jf, k);
                    }
                    if (turb)
                        for (int q = 0; q < NELEM(BC_TURB); q++) {
                            const int F_ = BC_TURB[q];
                            X(m, F_, i, r, k) = smax(BC_TURB_FLOOR[q], X(m, F_, i, jf, k));
                            X(m, F_, i, jm - 1 - r, k) = smax(BC_TURB_FLOOR[q], X(m, F_, i, jm - 1 - jf, k));
                        }
                }
            }
            for (int q = 0; q < NELEM(BC_THETA_ZERO); q++) {
                X(m, BC_THETA_ZERO[q], i, 0, k) = 0.0;
                X(m, BC_THETA_ZERO[q], i, jm - 1, k) = 0.0;
            }
            for (int q = 0; q < NELEM(BC_THETA_EXTRAP); q++) {
                const int F_ = BC_THETA_EXTRAP[q];
                X(m, F_, i, 0, k) = bc_form(form, X(m, F_, i, 1, k), X(m, F_, i, 2, k), X(m, F_, i, 3, k));
                X(m, F_, i, jm - 1, k) = bc_form(form, X(m, F_, i, jm - 2, k), X(m, F_, i, jm - 3, k), X(m, F_, i, jm - 4, k));
            }
            if (turb)
                for (int q = 0; q < NELEM(BC_TURB); q++) {
                    const int F_ = BC_TURB[q];
                    X(m, F_, i, 0, k) = smax(BC_TURB_FLOOR[q], c43 * X(m, F_, i, 1, k) - c13 * X(m, F_, i, 2, k));
                    X(m, F_, i, jm - 1, k) = smax(BC_TURB_FLOOR[q], c43 * X(m, F_, i, jm - 2, k) - c13 * X(m, F_, i, jm - 3, k));
                }
        }
    }
}

static void bc_phi(M* m) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int turb = p->turb_active;
    /* the phi list is the radius list (same fields) */
    #pragma omp parallel for
    for (int i = 0; i < im; i++) {
        for (int j = 0; j < jm; j++) {
            for (int q = 0; q < NELEM(BC_RADIUS); q++) {
                const int F_ = BC_RADIUS[q];
                if (p->phi_periodic) X(m, F_, i, j, km - 1) = X(m, F_, i, j, 0);
                else {
                    const double lo = c43 * X(m, F_, i, j, 1) - c13 * X(m, F_, i, j, 2);
                    const double hi = c43 * X(m, F_, i, j, km - 2) - c13 * X(m, F_, i, j, km - 3);
                    X(m, F_, i, j, 0) = X(m, F_, i, j, km - 1) = 0.5 * (lo + hi);
                }
            }
            if (turb)
                for (int q = 0; q < NELEM(BC_TURB); q++) {
                    const int F_ = BC_TURB[q];
                    if (p->phi_periodic) X(m, F_, i, j, 0) = X(m, F_, i, j, km - 1) = smax(BC_TURB_FLOOR[q], X(m, F_, i, j, 0));
                    else {
                        const double lo = c43 * X(m, F_, i, j, 1) - c13 * X(m, F_, i, j, 2);
                        const double hi = c43 * X(m, F_, i, j, km - 2) - c13 * X(m, F_, i, j, km - 3);
                        X(m, F_, i, j, 0) = X(m, F_, i, j, km - 1) = smax(BC_TURB_FLOOR[q], 0.5 * (lo + hi));
                    }
                }
        }
    }
}

static inline double rho_at(const M* m, int i, int j, int k) {
    if (!m->p->local_rho) return m->p->r_mix;
    const double rho = X(m, ATSAT_F_RHO_MIX, i, j, k);
    return (rho > 0.0 && isfinite(rho)) ? rho : m->p->r_mix;
}

static void bc_radius(M* m) {
    const atsat_dyn_params* p = m->p;
    const int im = m->im, jm = m->jm, km = m->km;
    const double c43 = 4.0 / 3.0, c13 = 1.0 / 3.0;
    const int form = p->bc_radius_form, bform = p->bc_bottom_form;
    const int turb = p->turb_active;
    const int k_lo = p->phi_periodic ? 0 : 1;
    #pragma omp parallel for
    for (int j = 1; j < jm - 1; j++) {
        for (int k = k_lo; k < km - 1; k++) {
            for (int q = 0; q < NELEM(BC_RADIUS); q++) {
                const int F_ = BC_RADIUS[q];
                const int fb = (bform != 0 && F_ != ATSAT_F_U) ? bform : form;
                X(m, F_, 0, j, k) = bc_form(fb, X(m, F_, 1, j, k), X(m, F_, 2, j, k), X(m, F_, 3, j, k));
                X(m, F_, im - 1, j, k) = bc_form(form, X(m, F_, im - 2, j, k), X(m, F_, im - 3, j, k), X(m, F_, im - 4, j, k));
            }
            if (turb)
                for (int q = 0; q < NELEM(BC_TURB); q++) {
                    const int F_ = BC_TURB[q];
                    X(m, F_, 0, j, k) = smax(BC_TURB_FLOOR[q], c43 * X(m, F_, 1, j, k) - c13 * X(m, F_, 2, j, k));
                    X(m, F_, im - 1, j, k) = smax(BC_TURB_FLOOR[q], c43 * X(m, F_, im - 2, j, k) - c13 * X(m, F_, im - 3, j, k));
                }
        }
    }
    if (p->bc_lid_u) {
        #pragma omp parallel for
        for (int j = 0; j < jm; j++)
            for (int k = 0; k < km; k++) { X(m, ATSAT_F_U, 0, j, k) = 0.0; X(m, ATSAT_F_U, im - 1, j, k) = 0.0; }
    }
    if (p->bc_top_taper) {
        const int iml = im - 1;
        #pragma omp parallel for
        for (int j = 0; j < jm; j++) {
            for (int k = 0; k < km; k++) {
                X(m, ATSAT_F_V, iml, j, k) = 0.0;
                X(m, ATSAT_F_W, iml, j, k) = 0.0;
                if (p->bc_top_taper == 2) {
                    X(m, ATSAT_F_V, iml - 1, j, k) = (1.0 / 3.0) * X(m, ATSAT_F_V, iml - 3, j, k);
                    X(m, ATSAT_F_W, iml - 1, j, k) = (1.0 / 3.0) * X(m, ATSAT_F_W, iml - 3, j, k);
                    X(m, ATSAT_F_V, iml - 2, j, k) = (2.0 / 3.0) * X(m, ATSAT_F_V, iml - 3, j, k);
                    X(m, ATSAT_F_W, iml - 2, j, k) = (2.0 / 3.0) * X(m, ATSAT_F_W, iml - 3, j, k);
                } else {
                    X(m, ATSAT_F_V, iml - 1, j, k) *= (1.0 / 3.0);
                    X(m, ATSAT_F_W, iml - 1, j, k) *= (1.0 / 3.0);
                    X(m, ATSAT_F_V, iml - 2, j, k) *= (2.0 / 3.0);
                    X(m, ATSAT_F_W, iml - 2, j, k) *= (2.0 / 3.0);
                }
            }
        }
    }
    /* BC_Sat::bcRadius, BC_Sat.cpp:61-105 */
    const int lid_copy = p->bc_species_lid_copy, wall_copy = p->bc_species_wall_copy;
    if (lid_copy == 0 && wall_copy == 0) return;
    #pragma omp parallel for
    for (int j = 0; j < jm; j++)
        for (int k = 0; k < km; k++) {
            const double fr = (wall_copy == 2) ? rho_at(m, 0, j, k) / rho_at(m, 1, j, k) : 1.0;
            for (int q = 0; q < NELEM(BC_SPECIES); q++) {
                const int F_ = BC_SPECIES[q];
                if (lid_copy != 0) X(m, F_, im - 1, j, k) = X(m, F_, im - 2, j, k);
                if (wall_copy != 0) X(m, F_, 0, j, k) = X(m, F_, 1, j, k) * fr;
            }
        }
}

/* ---------------- exported entry points ---------------- */

static int setup(M* m, const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields,
                 const double* vbar0, const double* ubar0, const double* p_baro, double* buoy) {
    if (!g || !p || !fields || g->im < 4 || g->jm < 5 || g->km < 4) return ATSAT_DYN_E_INVALID;
    if (p->chrom || p->cp_h2_dyn || p->print_diag) return ATSAT_DYN_E_UNSUPPORTED;
    memset(m, 0, sizeof(*m));
    m->im = g->im; m->jm = g->jm; m->km = g->km;
    m->rad_z = g->rad_z; m->the_z = g->the_z;
    m->dr = g->dr; m->dthe = g->dthe; m->dphi = g->dphi;
    m->p = p; m->f = fields;
    m->vbar0 = vbar0; m->ubar0 = ubar0; m->p_baro = p_baro;
    m->buoy = buoy;
    return ATSAT_DYN_OK;
}

int orc_buoyancy_ref_level(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, double* buoy) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, buoy);
    if (rc) return rc;
    buoyancy_ref_level(&m);
    return 0;
}

int orc_metric_pressure(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, const double* p_baro) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, p_baro, NULL);
    if (rc) return rc;
    metric_pressure(&m);
    return 0;
}

/* buoyancy level + p_metric + one RHS pass, as ref_harness "rhs" */
int orc_rhs(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, const double* vbar0,
            const double* ubar0, const double* p_baro, double* buoy) {
    M m; int rc = setup(&m, g, p, fields, vbar0, ubar0, p_baro, buoy);
    if (rc) return rc;
    buoyancy_ref_level(&m);
    if (p->metric_split) metric_pressure(&m);
    rhs_pass(&m);
    return 0;
}

int orc_rk4_step(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, const double* vbar0,
                 const double* ubar0, const double* p_baro, double* buoy) {
    M m; int rc = setup(&m, g, p, fields, vbar0, ubar0, p_baro, buoy);
    if (rc) return rc;
    const size_t n = (size_t)g->im * g->jm * g->km;
    for (int q = 0; q < ATSAT_NPROG; q++) {
        m.acc[q] = (double*)calloc(n, sizeof(double));
        if (!m.acc[q]) { for (int r = 0; r < q; r++) free(m.acc[r]); return ATSAT_DYN_E_NOMEM; }
    }
    rk4_step(&m);
    for (int q = 0; q < ATSAT_NPROG; q++) free(m.acc[q]);
    return 0;
}

int orc_mixture_density(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    mixture_density(&m);
    return 0;
}

int orc_prepare_projection_boundaries(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    prepare_projection_boundaries(&m, p->rigid_lid);
    return 0;
}

int orc_pressure(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, atsat_dyn_pstats* st) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    pressure(&m, st);
    return 0;
}

int orc_damp_wiggles(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, int fid, int along_i,
                     int along_j, int along_k, double strength, int passes) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    if (fid < 0 || fid >= ATSAT_NFIELDS) return ATSAT_DYN_E_INVALID;
    damp_wiggles(&m, fid, along_i, along_j, along_k, strength, passes);
    return ATSAT_DYN_OK;
}

int orc_damp_pdyn(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    damp_pdyn(&m);
    return ATSAT_DYN_OK;
}

int orc_clamp_negative_species(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields, double* budget) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    clamp_negative_species(&m, budget);
    return ATSAT_DYN_OK;
}

int orc_turbulence(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields,
                   const atsat_dyn_turb_params* tp, double* prod, double* vel_star) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    if (!tp || !prod || !vel_star || tp->model < 0 || tp->model > 2) return ATSAT_DYN_E_INVALID;
    turbulence_run(&m, tp, prod, vel_star);
    return ATSAT_DYN_OK;
}

int orc_restore_var(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    restore_var(&m);
    return 0;
}

int orc_boundary_conditions(const atsat_dyn_grid* g, const atsat_dyn_params* p, double** fields) {
    M m; int rc = setup(&m, g, p, fields, NULL, NULL, NULL, NULL);
    if (rc) return rc;
    bc_theta(&m);
    bc_phi(&m);
    bc_radius(&m);
    return 0;
}
