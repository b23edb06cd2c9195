// Shared definitions of the GB300 dynamical core: device layout, per-column geometry, the
// constants the kernels read, and the kernel entry points each translation unit provides.
//
// Device layout: structure of arrays, one pitched 3-D block per field, phi (k) innermost.
// A row (i, j) holds kp >= km values, kp a multiple of 32 so that every row starts on a 256-byte
// boundary for doubles and a 128-byte boundary for floats; element (i, j, k) sits at
// (i * jm + j) * kp + k. The radial planes are outermost.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/atsat_dyn.h"

namespace atsat {

constexpr int NPROG = ATSAT_NPROG;

// Per-(i,j) metric factors of one column. The RK members follow the CellGeometry that
// RungeKuttaSat builds (RungeKutta_Sat_Turb.cpp:223-243) plus the (i,j)-only products of RHSSat
// (Coriolis / centrifugal coefficients, RHS_Sat_Turb.cpp:310-350; v_metric :436); the P members are
// the pressure stencil weights (PressureSolver.h:349-353 for the sweep, :255-259 for lc_old).
struct alignas(16) ColGeo {
    double rm, inv_rm, inv_rm2, inv_rmsinthe;
    double inv_rm2sinthe, inv_rm2sinthe2, costhe_inv_rm2sinthe, cotanthe;
    double costhe, two_inv_rm, v_metric, exp_rm;
    double exp_2_rm, cor_rad, cor_the, cor_phi;      // cor_* multiply w, w, (cos v + sin u)
    double sinthe_true, cent_rad, cent_the, vbar0;
    double ubar0, p_num1, p_num2, p_num3;            // sweep weights
    double p_den, lc_num1, lc_num2, lc_num3;         // sweep denominator, lc_old weights
    double p_exp_rm, p_inv_rm, p_inv_rmsinthe, p_pad_cot_rm; // divergence-source factors; cot / rm
};
static_assert(sizeof(ColGeo) == 32 * 8, "ColGeo layout");

// Grid-wide constants, every one formed on the host in the reference's own expression order.
struct KConst {
    int im, jm, km, kp;
    int64_t plane;                 // jm * kp
    int64_t fsz;                   // im * jm * kp
    int periodic, turb, metric_split, coriolis_split;
    int adiabatic, adiabatic_rho, buoy_legacy, hydro_buoy;
    int t_limiter, cell_hold, rad_on, precip_on;
    int tmf_on, divu_on, press_incr, press_src;
    int rigid_lid, press_wall, pad_i0, pad_i1;
    double dr;
    double inv_2dr, inv_2dthe, inv_2dphi, inv_dr2, inv_dthe2, inv_dphi2;
    double coeff_energy_p;         // u_0 u_0 / (cp_mix t_ref)
    double to_nd;                  // 1 / (r_mix u_0 u_0 1e-5)
    double r_mix;
    double rR, t_ref, g;           // r_mix R_mix, for the buoyancy b = g p / (rR t t_ref)
    double kbuoy;                  // -nd_buoy * buoy_scale * buoyancy
    double legacy_buoy;            // buoyancy * g
    double inv_re, inv_re_pr;
    double inv_sc_re_ch4, inv_sc_re_h2o, inv_sc_re_h2s, inv_sc_re_nh3, inv_sc_re_nh4sh;
    double inv_sig_k, inv_sig_w;
    double turb_coupling, inv_pr_t;
    double Coriolis, centrifugal, chem;
    double metric_on, cor_rad_on;
    double rad_coupling, rad_num, rad_den_c;   // L_rad; cp_mix u_0 t_ref
    double precip_coupling, precip_num, precip_den;
    double tmf_chem;               // thermal_massflux * chemical_reaction
    double species_divu;
    double tke_max, dis_min;
    double dt;
    double pdyn_cap;
    double c43, c13;
};

// One precision's view of the fields a stage kernel touches.
template <typename T>
struct StageIO {
    const T* in[NPROG];            // stage input Y_s (stencil)
    T* out[NPROG];                 // next stage input Y_{s+1}, or y_{n+1} at the last stage
    const double* yn[NPROG];       // y_n
    double* acc[NPROG];            // running k1 + 2 k2 + 2 k3 + k4
    const T* p_dyn;
    const T* p_stat;
    const T* p_metric;
    const T* rho_mix;
    const T* nue;
    const T* q_precip;
    const T* q_rad;
    const T* tke_source;
    const T* dis_source;
    const T* s_precip[9];
    const T* massflux_h2s;
    const T* massflux_nh3;
    const T* massflux_nh4sh;
    const T* fluxlim_nh4sh;
    const T* thermalmassflux;
    double* rhs[NPROG];            // rhs_* (written where the mode asks for it)
    double* aux[3];                // aux_u/v/w
    const double* buoy;            // buoy_ref_level[im]
    const ColGeo* geo;             // [im * jm]
};

// ---- mixed precision (rk_mixed.cu) ----
constexpr int NCONV = 20;          // FP32 copies: rho_mix and the 19 point inputs nue .. thermalmassflux

// frozen FP32 fields formed in FP64 once per RK step
enum { FZ_DPR = 0, FZ_DPTH, FZ_DPPH, FZ_DPS, FZ_GU, FZ_GV, FZ_GW, FZ_BAN, FZ_BPS, NFZ };

// per-(i,j) geometry in FP32 for the stage kernel
struct alignas(16) ColGeoF {
    float inv_rm, inv_rm2, inv_rmsinthe, inv_rm2sinthe;
    float inv_rm2sinthe2, costhe_inv_rm2sinthe, cotanthe, costhe;
    float two_inv_rm, v_metric, sinthe_true, cor_the_c;     // cor_*_c include Coriolis and nd_cor
    float cor_phi_c, cor_rad_c, vbar0, ubar0;
};
static_assert(sizeof(ColGeoF) == 16 * 4, "ColGeoF layout");

struct MixedConstF {
    int im, jm, km, kp;
    int64_t plane;
    int metric_split, hydro_buoy, turb, rad_on;
    int precip_on, tmf_on, divu_on, pad0;
    float inv_2dr, inv_2dthe, inv_2dphi, inv_dr2, inv_dthe2, inv_dphi2;
    float coeff_energy_p, inv_re, inv_re_pr;
    float inv_sc_re_ch4, inv_sc_re_h2o, inv_sc_re_h2s, inv_sc_re_nh3, inv_sc_re_nh4sh;
    float inv_sig_k, inv_sig_w, turb_coupling, inv_pr_t;
    float chem, precip_coupling, precip_factor, rad_factor, r_mix;
    float tke_max, dis_min, species_divu, tmf_chem;
    float metric_on, cor_rad_on, kb, bref_scale;
    double tke_max_d, dis_min_d;
};

struct MixedIO {
    const float* yn32[NPROG];      // FP32 copy of y_n
    const float* wlo;              // y_n(w) - yn32(w)
    const float* dl_in[NPROG];     // stage increments; null entries: Y_s = y_n
    float* dl_out[NPROG];
    double* acc64[4];              // u, v, w, t
    float* acc32[NPROG - 4];       // the 13 scalars
    const double* yn64[NPROG];
    double* out64[NPROG];          // y_{n+1} (final stage)
    float* out32[NPROG];           // optional FP32 copy of y_{n+1}
    float* wlo_out;
    const float* fz[NFZ];
    const float* rho_mix;
    const float* nue;
    const float* q_precip;
    const float* q_rad;
    const float* tke_source;
    const float* dis_source;
    const float* s_precip[9];
    const float* massflux_h2s;
    const float* massflux_nh3;
    const float* massflux_nh4sh;
    const float* fluxlim_nh4sh;
    const float* thermalmassflux;
    double* rhs[NPROG];
    double* aux[3];
    const ColGeoF* geof;
    const double* buoy;
};

struct MixedPrep {
    int write_yn32;
    int skip_frozen;               // conversions only
    const double* yn64[NPROG];
    const double* live64[NPROG];
    float* yn32[NPROG];
    float* yn32_b[NPROG];          // optional second copy
    float* wlo;
    float* wlo_b;
    float* dl0[NPROG];             // null: not written
    const double* conv_src[NCONV];
    float* conv_dst[NCONV];
    int nconv;
    float* fz[NFZ];
    const double* p_dyn;
    const double* p_metric;
    const double* p_stat;
    const double* rho_mix;
    const double* buoy;
    const ColGeo* geo;
    double bnum;                   // g / (r_mix R_mix t_ref), or buoyancy g / (r_mix R_mix t_ref) legacy
};

enum StageMode {
    MODE_RHS = 0,       // tendencies only: all rhs_* and aux_*
    MODE_STAGE = 1,     // stages 0..2: acc and the next stage input
    MODE_FINAL = 2      // stage 3: acc, y_{n+1}, rhs_u/v/w and aux_u/v/w (all rhs_* if asked)
};

struct StageParams {
    int stage;
    int write_all_rhs;
    double c_in, wgt, sixth_dt;
};

// ---- kernel launchers (each returns cudaGetLastError()) ----
cudaError_t launch_rk_stage_fp64(const KConst& kc, const StageIO<double>& io, const StageParams& sp,
                                 int mode, cudaStream_t s);
cudaError_t launch_rk_stage_mixed(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode,
                                  cudaStream_t s);
cudaError_t launch_mixed_prepare(const KConst& kc, const MixedPrep& pr, cudaStream_t s);
cudaError_t launch_level_mean(const KConst& kc, const double* t, const double* p_stat,
                              const double* sin_j, double* partial, double* buoy, cudaStream_t s);
cudaError_t launch_metric_scan(const KConst& kc, const double* v, const double* w, const double* rm_tab,
                               const double* cor_j, const double* p_baro, double* p_metric, cudaStream_t s);
cudaError_t launch_density(const KConst& kc, const double* t, const double* p_stat, double R_mix,
                           double* rho, cudaStream_t s);
cudaError_t launch_projection_prep(const KConst& kc, double* const six[6], cudaStream_t s);
cudaError_t launch_press_source(const KConst& kc, const ColGeo* geo, const double* su, const double* sv,
                                const double* sw, const double* aux_u, const double* aux_v, const double* aux_w,
                                const double* rhs_u, const double* rhs_v, const double* rhs_w,
                                const double* p, double* src, unsigned long long* nclamp, cudaStream_t s);
cudaError_t launch_press_sweep(const KConst& kc, const ColGeo* geo, const double* src, double* p, int colour,
                               cudaStream_t s);
cudaError_t launch_press_boundary(const KConst& kc, double* p, cudaStream_t s);
cudaError_t launch_copy_fields(const KConst& kc, double* const* dst, const double* const* src, int n,
                               cudaStream_t s);
// s32 (may be null): FP32 copies to keep in step, indexed by field id; wlo: the second FP32 word of w.
cudaError_t launch_boundary_conditions(const KConst& kc, const atsat_dyn_params& p, double* const* f,
                                       float* const* s32, float* wlo, cudaStream_t s);
cudaError_t launch_count_nonfinite(const KConst& kc, const double* x, unsigned long long* count,
                                   cudaStream_t s);

}  // namespace atsat
