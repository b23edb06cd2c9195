// Shared definitions of the GB300 dynamical core: device layout, per-column geometry, the
// constants the kernels read, and the kernel entry points each translation unit provides.
//
// Device layout: structure of arrays, one pitched 3-D block per field, phi (k) innermost.
// A row (i, j) holds kp >= km values, kp a multiple of 32 so that every row starts on a 256-byte
// boundary for doubles and a 128-byte boundary for floats; element (i, j, k) sits at
// (i * jm + j) * kp + k. The radial planes are outermost.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/atsat_dyn.h"

namespace atsat {

constexpr int NPROG = ATSAT_NPROG;

// ---- binary32 <-> binary64 conversions on the integer pipe ----
// GB300 runs F2F (float <-> double) on its FP64 pipe, two operations per SM per cycle like a DADD.
// These rebuild the IEEE-754 encodings with integer operations for the common cases -- normal
// numbers and zeros -- and defer to the hardware conversion for subnormals, infinities and NaNs.
// Both give the hardware's bits (round to nearest even for the narrowing).
// The rare cases go through calls that the compiler cannot if-convert: an inlined fallback would be
// evaluated (and its F2F issued) on every call.
static __device__ __noinline__ double f2d_rare(float f) { return (double)f; }
static __device__ __noinline__ float d2f_rare(double d) { return (float)d; }

// The double's two words pass through a register move in inline PTX: tests on its bits then stay
// integer tests (the compiler would otherwise fold a test such as "all bits but the sign are zero"
// back into an FP64 comparison, a DSETP on the FP64 pipe).
__device__ __forceinline__ void split_f64(double d, uint32_t& lo, uint32_t& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(d));
}
__device__ __forceinline__ double join_f64(uint32_t lo, uint32_t hi) {
    double d;
    asm("mov.b64 %0, {%1, %2};" : "=d"(d) : "r"(lo), "r"(hi));
    return d;
}

__device__ __forceinline__ double f2d(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t a = b & 0x7FFFFFFFu;
    if (a - 0x00800000u < 0x7F000000u)            // biased exponent 1..254
        return join_f64(a << 29, (b & 0x80000000u) | ((a >> 3) + (896u << 20)));
    if (a == 0u) return join_f64(0u, b);
    return f2d_rare(f);
}

__device__ __forceinline__ float d2f(double d) {
    uint32_t lo, hi;
    split_f64(d, lo, hi);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e - 897u < 254u) {                         // result exponent 1..254 before rounding
        uint32_t q = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
        const uint32_t r = lo & 0x1FFFFFFFu;
        q += (r > 0x10000000u || (r == 0x10000000u && (q & 1u))) ? 1u : 0u;   // a carry into 255 is inf
        return __uint_as_float(q | (hi & 0x80000000u));
    }
    if (((hi << 1) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    return d2f_rare(d);
}

// 1/x for x > 0 in FP32's normal range: the FP32 reciprocal refined by one Newton-Raphson step
// r <- r + r (1 - x r) (relative error 2^-23 -> ~2^-46, always from below). in_range tests the range on
// the integer pipe (exponent field of x); x's FP32 copy and the result's widening are integer too.
__device__ __forceinline__ bool in_rcp_range(double x) {
    uint32_t lo, hi;
    split_f64(x, lo, hi);
    return (hi >> 31) == 0u && ((hi >> 20) & 0x7FFu) - 897u < 250u;   // 0 < x, float-normal with margin
}
__device__ __forceinline__ double recip_nr(double x) {
    const double r = f2d(__frcp_rn(d2f(x)));
    return fma(r, fma(-x, r, 1.0), r);
}

// a / b with b's reciprocal refined as above where b is in range (relative error ~2^-46 instead of the
// division's half ulp, at three FP64 operations instead of about a dozen); the division elsewhere
__device__ __forceinline__ double qdiv(double a, double b) { return in_rcp_range(b) ? a * recip_nr(b) : a / b; }

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
    // the source factors times the centred-difference scales (exp_rm / (2 dr), 1 / (2 dthe rm),
    // 1 / (2 dphi rm sin)) and 1 / p_den: one product per term instead of two, no FP64 division
    double src_r, src_the, src_phi, p_inv_den;
    // the FP64 stage's stencil scales folded into one coefficient per term (raw differences a0 = f(i+1) -
    // f(i-1), b0, c0 along theta and phi, second differences a1, b1, c1): transport v b0 t_the + w c0 t_phi,
    // diffusion a0 d_r1 + b1 d_t2 + b0 d_t1 + c1 d_p2, and the cross terms of the u, v, w diffusion
    double t_the, t_phi, d_r1, d_t2, d_t1, d_p2, x_v1, x_v2, x_w1, pad_c;
};
static_assert(sizeof(ColGeo) == 46 * 8, "ColGeo layout");

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
    double buoy_c;                 // g / (rR t_ref)
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
    int precip_on, tmf_on, divu_on, fsz_over_int;   // fsz_over_int: cell offsets need 64 bits
    float inv_2dr, inv_2dthe, inv_2dphi, inv_dr2, inv_dthe2, inv_dphi2;
    float coeff_energy_p, inv_re, inv_re_pr;
    float inv_sc_re_ch4, inv_sc_re_h2o, inv_sc_re_h2s, inv_sc_re_nh3, inv_sc_re_nh4sh;
    float inv_sig_k, inv_sig_w, turb_coupling, inv_pr_t;
    float chem, precip_coupling, precip_factor, rad_factor, r_mix;
    float tke_max, dis_min, species_divu, tmf_chem;
    float metric_on, cor_rad_on, kb, bref_scale;
    double tke_max_d, dis_min_d;
};

// The stage increments are dl_s = c_in k_{s-1} (stage inputs Y_s = y_n + dl_s). Stages 0..2 write
// dl_1 = dt/2 k1, dl_2 = dt/2 k2, dl_3 = dt k3, so that the final stage forms
// y_{n+1} = y_n + (dl_1 + 2 dl_2 + dl_3) / 3 + dt/6 k4 without running sums; tke and dis, whose
// increments are clamped, keep a running k1 + 2 k2 + 2 k3 instead.
struct MixedIO {
    const float* yn32[NPROG];      // FP32 copy of y_n
    const float* wlo;              // y_n(w) - yn32(w)
    const float* dl_in[NPROG];     // stage increments; null entries: Y_s = y_n
    float* dl_out[NPROG];          // stages 0..2
    float* dl1[NPROG];       // final stage: dl_1 and dl_2
    const float* dl2[NPROG];
    float* acc_turb[2];            // tke, dis
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

// per-column constants of the prepare kernel (products formed on the host)
struct alignas(16) PrepGeo {
    double s_the;                  // inv_2dthe / rm
    double cot_rm;                 // cot(theta) / rm
    double cor_the_c;              // Coriolis * cor_the
    double cent_the_c;             // centrifugal * cent_the
    double cent_rad_c;             // centrifugal * cent_rad
    double cor_rad_c;              // cor_rad_on * Coriolis * cor_rad
    double metric_inv_rm;          // metric_on / rm
    float s_the_f, s_phi_f;        // inv_2dthe / rm, inv_2dphi / (rm sin theta) in FP32
};
static_assert(sizeof(PrepGeo) == 64, "PrepGeo layout");

struct MixedPrep {
    int write_yn32;                // yn32[q] (where non-null) and wlo from yn64
    int any_dl0;                   // some dl0[0][q] is non-null
    int skip_frozen;               // conversions only
    const double* yn64[NPROG];
    const double* live64[NPROG];
    float* yn32[NPROG];
    float* yn32_b[NPROG];          // optional second copy
    float* wlo;
    float* wlo_b;
    float* dl0[3][NPROG];          // live - y_n into each increment buffer (null: not written)
    const double* conv_src[NCONV];
    float* conv_dst[NCONV];
    int nconv;
    float* fz[NFZ];
    const double* p_dyn;
    const double* p_metric;
    const double* p_stat;
    const double* rho_mix;
    const double* buoy;
    const PrepGeo* pgeo;
    double bnum;                   // g / (r_mix R_mix t_ref), or buoyancy g / (r_mix R_mix t_ref) legacy
    float bnum_f, inv_2dr_f, dps_scale_f, r_mix_f;
    int cor_rad;                   // the radial Coriolis term is on (coriolis_split off)
};

// The TMA-tiled stage kernel: the FP32 arrays live in one slab at a fixed stride, addressed by a 4-D
// tensor map (k, j, i, array); `item` lists the arrays the kernel streams, in the order it reads them.
// A block integrates TILE_K x TILE_J x TILE_I cells (k, j, i); its box carries a halo of one cell in
// j and i and of four in k (the tensor copy's innermost coordinate must be a multiple of 16 bytes).
// The seam box fetches the periodic partner column (k = km-2 for k = 0, k = 0 for k = km-2) when the
// main box does not hold it.
constexpr int TILE_K = 32, TILE_J = 8, TILE_I = 2;
constexpr long long TILE_WAIT_LIMIT = 1LL << 31;   // SM clocks (about a second) before a bounded wait gives up
constexpr int TILE_BX = TILE_K + 8, TILE_BY = TILE_J + 2, TILE_BZ = TILE_I + 2;
constexpr int TILE_SEAM_X = 4;
constexpr int TILE_MAX_ITEMS = 2 * NPROG + 1;
// the tracer kernel's taller tile: four radial levels per thread
constexpr int TTILE_I = 4, TTILE_BZ = TTILE_I + 2;
struct TilePlan {
    int n_items;
    int item[TILE_MAX_ITEMS];
    int arr_yn[NPROG];             // tensor-map array index of each stencil array (-1: absent)
    int arr_dl[NPROG];
    int arr_lo;
    unsigned int* err;             // device status word: bit 0 producer wait, bit 1 consumer wait, bit 2 plan
    long long wait_limit;          // SM clocks before a bounded wait gives up
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
    float c_in_f, wgt_f, sixth_dt_f;
};

// ---- kernel launchers (each returns cudaGetLastError()) ----
cudaError_t launch_rk_stage_fp64(const KConst& kc, const StageIO<double>& io, const StageParams& sp,
                                 int mode, cudaStream_t s);
cudaError_t launch_rk_stage_mixed(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode,
                                  cudaStream_t s);
cudaError_t launch_mixed_prepare(const KConst& kc, const MixedPrep& pr, cudaStream_t s);
// momentum / temperature kernel, then the tracer kernel with `groups` (1, 3 or 13) threads per cell
cudaError_t launch_rk_split(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode, int groups,
                            cudaStream_t s);
// tensor maps are CUtensorMap objects (128 bytes), passed opaquely
struct TileMaps {
    alignas(64) unsigned char main[128];    // box TILE_BX x TILE_BY x TILE_BZ
    alignas(64) unsigned char seam[128];    // box TILE_SEAM_X x TILE_J x TILE_I
    alignas(64) unsigned char main4[128];   // box TILE_BX x TILE_BY x TTILE_BZ
    alignas(64) unsigned char seam4[128];   // box TILE_SEAM_X x TILE_J x TTILE_I
    alignas(64) unsigned char pt4[128];     // box TILE_K x TILE_J x TTILE_I (point values, no halo)
    alignas(64) unsigned char pt2[128];     // box TILE_K x TILE_J x TILE_I (point values, no halo)
    alignas(64) unsigned char plane1[128];  // box TILE_BX x TILE_BY x 1: one radial plane with its halo
    alignas(64) unsigned char seam1[128];   // box TILE_SEAM_X x TILE_J x 1
    alignas(64) unsigned char pt1[128];     // box TILE_K x TILE_J x 1
};

// The tracer kernel's stream: every array it reads, in consumption order, each either a halo box
// (kind 0) or a point box (kind 1).
constexpr int TRACER_MAX_ITEMS = 96;
struct TracerPlan {
    int n_items;
    int arr[TRACER_MAX_ITEMS];
    unsigned char kind[TRACER_MAX_ITEMS];
    unsigned int* err;
    long long wait_limit;          // SM clocks before a consumer's or the producer's slot wait gives up
    int withhold;                  // test hook: the producer leaves the last `withhold` items unissued
};
cudaError_t launch_rk_tile(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                           const TilePlan& plan, int mode, cudaStream_t s);
size_t rk_tile_smem_bytes();
// the 13 tracer fields alone, TMA-tiled (after rk_mom_kernel; species_divu off)
cudaError_t launch_rk_tracer_tile(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io,
                                  const StageParams& sp, const TracerPlan& plan, int mode, cudaStream_t s);
cudaError_t launch_rk_mom(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode, cudaStream_t s);
int tracer_plan_items(int mode, bool has_dl, bool turb);
// the momentum / temperature equations alone, TMA-tiled (species_divu off)
cudaError_t launch_rk_mom_tile(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                               const TracerPlan& plan, int mode, cudaStream_t s);
int mom_plan_items(bool has_dl);

// The radial-march momentum / temperature kernel (rk_mom_march.cu, species_divu off): a block owns
// TILE_K x TILE_J columns (k, j) and walks `levels` radial levels; per level its producer streams one plane
// (with its theta / phi halo) of each stencil array and the level's point inputs, and the consumers keep
// the stencil's radial neighbours in registers. Point items per level, in this order: nue, the frozen DPR,
// GU, BAN, BPS, DPTH, GV, DPPH, GW, DPS, then the optional ones at the positions below.
constexpr int MARCH_MAX_PT = 22;
struct MarchPlan {
    int n_halo;                    // stencil arrays: u_yn [u_dl] v_yn [v_dl] w_yn w_lo [w_dl] t_yn [t_dl]
    int halo[9];
    int n_pt;
    int pt[MARCH_MAX_PT];
    int p_qprecip, p_rho, p_qrad, p_tmf;   // positions of the optional point items (-1: absent)
    int p_dl;                      // final stage: dl_1, dl_2 of u, v, w, t from here on (-1: other stages)
    int levels;                    // radial levels per block
    unsigned int* err;
    long long wait_limit;
    int withhold;                  // test hook: the producer leaves the last `withhold` level groups unissued
    int compact;                   // intermediate stages with at most 12 point arrays: three blocks per SM
};
cudaError_t launch_rk_mom_march(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                                const MarchPlan& plan, int mode, cudaStream_t s);

// standalone pressure-equation solver (poisson.cu)
struct PoissonSolver;
PoissonSolver* poisson_create(const KConst& kc, const ColGeo* geo_dev, const std::vector<ColGeo>& geo_h,
                              cudaStream_t s, std::string* err);
void poisson_destroy(PoissonSolver* P);
double* poisson_f(PoissonSolver* P);          // device source (pitched)
double* poisson_p(PoissonSolver* P);          // device solution (pitched)
const std::vector<double>& poisson_null_vector(PoissonSolver* P);   // [(j-1) * (im-2) + (i-1)]
void poisson_sweep_stats(PoissonSolver* P, int* sweeps_per_pass, double* sweep_ms);
cudaError_t poisson_run(PoissonSolver* P, int method, double tol, int max_iter, int inner, double omega,
                        int* iters, int* inner_total, double* rel);
cudaError_t launch_level_mean(const KConst& kc, const double* t, const double* p_stat,
                              const double* sin_j, double* partial, double* buoy, cudaStream_t s);
cudaError_t launch_metric_scan(const KConst& kc, const double* v, const double* w, const double* inv_rm,
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

// the driver's glue (glue.cu): one axis of AtomUtils::damp_wiggles; cSaturnModel::clampNegativeSpecies
cudaError_t launch_damp_axis(const KConst& kc, const double* tmp, double* f, double coeff, int axis, int seam,
                             cudaStream_t s);
// the species floor; `partial` holds clamp_partial_doubles() doubles of per-block sums
size_t clamp_partial_doubles();
cudaError_t launch_clamp_species(const KConst& kc, double* const f[11], float* const s32[11], double* added,
                                 unsigned long long* cells, double* partial, cudaStream_t s);

// the final stage's FP64 half of fields q0..q1 after a tiled stage kernel (rk_mixed.cu)
cudaError_t launch_final_combine(const MixedConstF& kf, const MixedIO& io, int q0, int q1, cudaStream_t s);
cudaError_t launch_nonfinite_fields(const KConst& kc, const double* const* f, int n, unsigned long long* count,
                                    cudaStream_t s);

// Turbulence<cSaturnModel>::run (turbulence.cu). Device tables per level i and row j, formed on the host with
// the reference's expressions; height_m / thick_m from the model's float layer table.
struct TurbTables {
    const double *rm, *inv_rm, *inv_rm2dthe, *height_m, *thick_m;   // im
    const double *sinthe, *cotanthe;                                // jm: exact-zero guard, no floor
    const double* inv_rmsinthe2dphi;                                // im x jm
    double dr, dthe, dphi, taper_dz;
};
cudaError_t launch_turbulence(const KConst& K, const atsat_dyn_params& p, const atsat_dyn_turb_params& tp,
                              const TurbTables& tab, double* const* f, double* prod, double* vel_star, cudaStream_t s,
                              int* launches);

// PRESS_LINE / PRESS_BAROTROPIC (press_variants.cu)
struct BaroTables {
    double A2;                                    // sum over i = 1..im-2 of 1 / rm^2
    const double *ct, *st;                        // (N/2 + 1) x N: cos, sin(2 pi (m k mod N) / N)
    const double *lam, *sinthe, *abs_sin;         // per mode; the solver's sine table (jm); |sin(theta_j+1)|
    double *R, *ra, *Ac, *As, *cp, *dp;           // scratch
};
cudaError_t launch_line_pass(const KConst& kc, const ColGeo* geo, const double* src, double* p, double* cpb,
                             double* dpb, int colour, cudaStream_t s, int* launches);
cudaError_t launch_interior_mean(const KConst& kc, const double* p, double* partial, double* out, cudaStream_t s,
                                 int* launches);
int interior_mean_partials(const KConst& kc);
cudaError_t launch_mean_shift(const KConst& kc, double* p, const double* mean, cudaStream_t s);
cudaError_t launch_barotropic(const KConst& kc, const ColGeo* geo, const double* src, double* p, const BaroTables& T,
                              cudaStream_t s, int* launches);
cudaError_t launch_copy_fields(const KConst& kc, double* const* dst, const double* const* src, int n,
                               cudaStream_t s);
// s32 (may be null): FP32 copies to keep in step, indexed by field id; wlo: the second FP32 word of w.
cudaError_t launch_boundary_conditions(const KConst& kc, const atsat_dyn_params& p, double* const* f,
                                       float* const* s32, float* wlo, cudaStream_t s);
// a host binding moved by the SMs (host_xfer.cu): a contiguous array (`base`, rows of km doubles) or a
// device-resident table of row pointers (`rows`), and the device field (rows of kp doubles)
constexpr int HOST_BATCH_MAX = 64;
struct HostField {
    double* base;
    double* const* rows;
    double* dev;
    float* dev32;                  // upload only: the field's FP32 copy, written from the same values (or null)
};
struct HostBatch {
    HostField f[HOST_BATCH_MAX];
    int n;
};
cudaError_t launch_host_transfer(const HostBatch& b, int to_device, int64_t nrows, int km, int kp, cudaStream_t s);
cudaError_t launch_repitch(double* dst, int dst_pitch, const double* src, int src_pitch, int width, int64_t rows,
                           cudaStream_t s);
cudaError_t launch_count_nonfinite(const KConst& kc, const double* x, unsigned long long* count,
                                   cudaStream_t s);

}  // namespace atsat
