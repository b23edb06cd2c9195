// Mixed-precision RK4 stage of the ATSAT dynamical core (RungeKuttaSat / RHSSat,
// planet/RungeKutta_Sat_Turb.cpp:110-387, planet/RHS_Sat_Turb.cpp:25-1016).
//
// Storage per prognostic field q:
//   yn64[q]  y_n in FP64 (the ABI's n-level field)
//   yn32[q]  an FP32 copy of y_n, read by the stencils
//   dl[q]    the stage input as an FP32 increment, Y_s = y_n + dl (dl = c_in * k_{s-1}; zero at stage 0
//            when the live state equals y_n)
//   acc[q]   k1 + 2 k2 + 2 k3 + k4 in FP64
// The derivatives of all 17 fields are taken in FP32 from yn32 + dl. The centre values of u, v, w and t
// are rebuilt in FP64 (yn64 + dl), and every term of the momentum equations that is large and cancels --
// the pressure and p_metric gradients, the buoyancy anomaly against the FP64 level mean, the Coriolis
// force of the zonal jet and its w^2 cot / r metric partner, the centrifugal force -- is formed and summed
// in FP64; the transport and diffusion terms (small against those) are FP32. The accumulator and the final
// y_{n+1} = y_n + dt/6 acc are FP64. The increments for the next stage are rounded to FP32 only after
// being formed: their rounding error is 6e-8 of dt * k, not of the field.
#include "dyn_common.cuh"

namespace atsat {

namespace {

struct D6f { float dr, d2r, dthe, d2the, dphi, d2phi; };

struct KF {          // FP32 copies of the grid constants
    float inv_2dr, inv_2dthe, inv_2dphi, inv_dr2, inv_dthe2, inv_dphi2;
};

__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldd(const double* p) { return __ldg(p); }

// Y_s at an offset: yn32 + dl (dl may be absent at stage 0)
__device__ __forceinline__ float ys(const float* __restrict__ yn, const float* __restrict__ dl, int64_t c) {
    return dl ? ldf(yn + c) + ldf(dl + c) : ldf(yn + c);
}

// Differences of Y_s = y_n + dl are taken on the two parts separately and then added: y_n's FP32 copy
// carries a fixed rounding of the field, dl the small increment at its own precision. Summing first would
// round the increment against the field (0.85 + 1e-5 loses the increment's low digits), and the stencil
// would difference that rounding noise.
__device__ __forceinline__ void diff7(const float* f, int64_t c, int64_t P, int kp, int dkw, int dke, float* e) {
    const float x = ldf(f + c);
    const float rp = ldf(f + c + P), rn = ldf(f + c - P);
    const float tp = ldf(f + c + kp), tn = ldf(f + c - kp);
    const float pe = ldf(f + c + dke), pw = ldf(f + c + dkw);
    e[0] = rp - rn;
    e[1] = rp - 2.0f * x + rn;
    e[2] = tp - tn;
    e[3] = tp - 2.0f * x + tn;
    e[4] = pe - pw;
    e[5] = pe - 2.0f * x + pw;
}

__device__ __forceinline__ void derivs32(const float* yn, const float* dl, int64_t c, int64_t P, int kp, int dkw,
                                         int dke, const KF& K, D6f& d) {
    float a[6];
    diff7(yn, c, P, kp, dkw, dke, a);
    if (dl) {
        float b[6];
        diff7(dl, c, P, kp, dkw, dke, b);
#pragma unroll
        for (int q = 0; q < 6; q++) a[q] += b[q];
    }
    d.dr = a[0] * K.inv_2dr;
    d.d2r = a[1] * K.inv_dr2;
    d.dthe = a[2] * K.inv_2dthe;
    d.d2the = a[3] * K.inv_dthe2;
    d.dphi = a[4] * K.inv_2dphi;
    d.d2phi = a[5] * K.inv_dphi2;
}

// The zonal wind w (|w| up to ~0.85, with small zonal variations) is differenced from its FP64 y_n: an
// FP32 copy would round w by 3e-8 independently per cell, and near the poles w * dw/dphi / (r sin theta)
// turns that rounding into a tendency error larger than the FP32 arithmetic of every other term.
__device__ __forceinline__ void derivs_wide(const double* yn, const float* dl, int64_t c, int64_t P, int kp,
                                            int dkw, int dke, const KF& K, D6f& d) {
    const double x = ldd(yn + c);
    const double rp = ldd(yn + c + P), rn = ldd(yn + c - P);
    const double tp = ldd(yn + c + kp), tn = ldd(yn + c - kp);
    const double pe = ldd(yn + c + dke), pw = ldd(yn + c + dkw);
    float a[6];
    a[0] = (float)(rp - rn);
    a[1] = (float)(rp - 2.0 * x + rn);
    a[2] = (float)(tp - tn);
    a[3] = (float)(tp - 2.0 * x + tn);
    a[4] = (float)(pe - pw);
    a[5] = (float)(pe - 2.0 * x + pw);
    if (dl) {
        float b[6];
        diff7(dl, c, P, kp, dkw, dke, b);
#pragma unroll
        for (int q = 0; q < 6; q++) a[q] += b[q];
    }
    d.dr = a[0] * K.inv_2dr;
    d.d2r = a[1] * K.inv_dr2;
    d.dthe = a[2] * K.inv_2dthe;
    d.d2the = a[3] * K.inv_dthe2;
    d.dphi = a[4] * K.inv_2dphi;
    d.d2phi = a[5] * K.inv_dphi2;
}

struct GeoF {
    float inv_rm, inv_rm2, inv_rmsinthe, inv_rm2sinthe, inv_rm2sinthe2, costhe_inv_rm2sinthe, cotanthe;
    float costhe, two_inv_rm, v_metric, sinthe_true;
};

__device__ __forceinline__ float transport32(float u, float v, float w, const D6f& d, const GeoF& g) {
    return u * d.dr + v * d.dthe * g.inv_rm + w * d.dphi * g.inv_rmsinthe;
}

__device__ __forceinline__ float diffusion32(const D6f& d, const GeoF& g) {
    return d.d2r + d.dr * g.two_inv_rm + d.d2the * g.inv_rm2 + d.dthe * g.costhe_inv_rm2sinthe
         + d.d2phi * g.inv_rm2sinthe2;
}

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smaxf(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float sminf(float a, float b) { return (b < a) ? b : a; }

template <int MODE>
__device__ __forceinline__ void emit(const MixedIO& io, const StageParams& sp, const KConst& K, int q, int64_t c,
                                     double r, float y32_for_clamp) {
    if (MODE == MODE_RHS) {
        io.rhs[q][c] = r;
        return;
    }
    if (MODE == MODE_STAGE) {
        const double a = (sp.stage == 0) ? sp.wgt * r : io.acc[q][c] + sp.wgt * r;
        io.acc[q][c] = a;
        float d;
        if (q == ATSAT_F_TKE || q == ATSAT_F_DIS) {
            // the clamps of the stage input (RungeKutta_Sat_Turb.cpp:311-316), on Y = y_n + c_in k
            const float y = y32_for_clamp + (float)(sp.c_in * r);
            const float yc = (q == ATSAT_F_TKE) ? sminf(smaxf(y, 0.0f), (float)K.tke_max) : smaxf(y, (float)K.dis_min);
            d = yc - y32_for_clamp;
        } else {
            d = (float)(sp.c_in * r);
        }
        io.dl_out[q][c] = d;
        return;
    }
    // final: y_{n+1} = y_n + dt/6 (acc + k4), FP64
    const double a = io.acc[q][c] + sp.wgt * r;
    double y = ldd(io.yn64[q] + c) + sp.sixth_dt * a;
    if (q == ATSAT_F_TKE) y = smin(smax(y, 0.0), K.tke_max);
    else if (q == ATSAT_F_DIS) y = smax(y, K.dis_min);
    io.out64[q][c] = y;
    if (io.out32[q]) io.out32[q][c] = (float)y;
    if (sp.write_all_rhs || q < 3) io.rhs[q][c] = r;
}

template <int MODE>
__global__ void __launch_bounds__(256) rk_stage_mixed_kernel(const KConst K, const KF KF_, const MixedIO io,
                                                             const StageParams sp) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const bool interior = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    const int64_t P = K.plane;
    const int kp = K.kp;
    const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
    if (!interior) {
        // Cells the step does not integrate keep Y_s = y_n + dl_0 at every stage: carry dl forward.
        if (MODE == MODE_STAGE) {
#pragma unroll 1
            for (int q = 0; q < NPROG; q++) io.dl_out[q][c] = io.dl_in[q] ? ldf(io.dl_in[q] + c) : 0.0f;
        }
        return;
    }
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const int dkw = kw - k, dke = ke - k;
    const float* const* dl = io.dl_in;
    auto dlq = [&](int q) -> const float* { return dl[q]; };

    const ColGeo* gp = io.geo + ((int64_t)i * K.jm + j);
    GeoF g;
    g.inv_rm = (float)ldd(&gp->inv_rm);
    g.inv_rm2 = (float)ldd(&gp->inv_rm2);
    g.inv_rmsinthe = (float)ldd(&gp->inv_rmsinthe);
    g.inv_rm2sinthe = (float)ldd(&gp->inv_rm2sinthe);
    g.inv_rm2sinthe2 = (float)ldd(&gp->inv_rm2sinthe2);
    g.costhe_inv_rm2sinthe = (float)ldd(&gp->costhe_inv_rm2sinthe);
    g.cotanthe = (float)ldd(&gp->cotanthe);
    g.costhe = (float)ldd(&gp->costhe);
    g.two_inv_rm = (float)ldd(&gp->two_inv_rm);
    g.v_metric = (float)ldd(&gp->v_metric);
    g.sinthe_true = (float)ldd(&gp->sinthe_true);
    const double inv_rm = ldd(&gp->inv_rm), inv_rmsinthe = ldd(&gp->inv_rmsinthe);

    // FP64 centre values of the momentum fields and the temperature
    auto centre = [&](int q) -> double {
        const double y = ldd(io.yn64[q] + c);
        return dlq(q) ? y + (double)ldf(dlq(q) + c) : y;
    };
    const double u = centre(ATSAT_F_U), v = centre(ATSAT_F_V), w = centre(ATSAT_F_W), t = centre(ATSAT_F_T);
    const float uf = (float)u, vf = (float)v, wf = (float)w;

    D6f du, dv, dw;
    derivs32(io.yn32[ATSAT_F_U], dlq(ATSAT_F_U), c, P, kp, dkw, dke, KF_, du);
    derivs32(io.yn32[ATSAT_F_V], dlq(ATSAT_F_V), c, P, kp, dkw, dke, KF_, dv);
    derivs_wide(io.yn64[ATSAT_F_W], dlq(ATSAT_F_W), c, P, kp, dkw, dke, KF_, dw);

    const double dpdr = (ldd(io.p_dyn + c + P) - ldd(io.p_dyn + c - P)) * K.inv_2dr;
    const double dpdthe = (ldd(io.p_dyn + c + kp) - ldd(io.p_dyn + c - kp)) * K.inv_2dthe;
    const double dpdphi = (ldd(io.p_dyn + c + dke) - ldd(io.p_dyn + c + dkw)) * K.inv_2dphi;

    const float nue_c = ldf(io.nue + c);
    const float nue_t = (K.turb_coupling != 0.0 && isfinite(nue_c)) ? (float)K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
    const float nue_t_s = nue_t * (float)K.inv_pr_t;
    const float inv_re = (float)K.inv_re;

    // ---- momentum ----
    {
        const double cor_the = ldd(&gp->cor_the) * w;
        // the zonal Coriolis force and the metric terms of the v and w equations are FP64: they are as
        // large as rhs_v / rhs_w themselves near the poles
        const double cot = ldd(&gp->cotanthe);
        const double cor_phi = ldd(&gp->cor_phi) * (ldd(&gp->costhe) * (v - ldd(&gp->vbar0))
                                                    + ldd(&gp->sinthe_true) * (u - ldd(&gp->ubar0)));

        const float tr_u = uf * du.dr + vf * du.dthe * g.inv_rm + wf * du.dphi * g.inv_rmsinthe;
        const float tr_v = uf * dv.dr + vf * dv.dthe * g.inv_rm + wf * dv.dphi * g.inv_rmsinthe;
        const float tr_w = uf * dw.dr + vf * dw.dthe * g.inv_rm + wf * dw.dphi * g.inv_rmsinthe;
        const double tr_v_metric = (u * v - w * w * cot) * inv_rm;
        const double tr_w_metric = (w * u + v * w * cot) * inv_rm;
        const float diffusion_u = du.d2r + 2.0f * uf * g.inv_rm2 + du.d2the * g.inv_rm2 + 4.0f * du.dr * g.inv_rm
                                + du.dthe * g.costhe_inv_rm2sinthe + du.d2phi * g.inv_rm2sinthe2;
        const float diffusion_v = dv.d2r + dv.dr * g.two_inv_rm + dv.d2the * g.inv_rm2
                                + dv.dthe * g.costhe_inv_rm2sinthe - g.v_metric * vf
                                + dv.d2phi * g.inv_rm2sinthe2 + 2.0f * du.dthe * g.inv_rm2
                                - dw.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
        const float diffusion_w = dw.d2r + dw.dr * g.two_inv_rm + dw.d2the * g.inv_rm2
                                + dw.dthe * g.costhe_inv_rm2sinthe - g.v_metric * wf
                                + dw.d2phi * g.inv_rm2sinthe2 + 2.0f * du.dphi * g.inv_rm2sinthe
                                + dv.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;

        double buoyancy_u = 0.0;
        if (t > 0.0 && !K.hydro_buoy) {
            const double ps = ldd(io.p_stat64 + c);
            if (K.buoy_legacy) buoyancy_u = K.legacy_buoy * (ps + ldd(io.p_dyn + c)) / (K.rR * t * K.t_ref);
            else buoyancy_u = K.kbuoy * (K.g * ps / (K.rR * t * K.t_ref) - ldd(io.buoy + i));
        }
        double metric_u = 0.0;
        if (!K.metric_split) metric_u = K.metric_on * (v * v + w * w) * inv_rm;
        const double rhs_u = -dpdr + buoyancy_u - (double)tr_u + metric_u
                           + (double)(diffusion_u * inv_re + diffusion_u * nue_t)
                           - K.cor_rad_on * K.Coriolis * (ldd(&gp->cor_rad) * w) + K.centrifugal * ldd(&gp->cent_rad);
        double dpmdthe = 0.0, dpmdphi = 0.0;
        if (K.metric_split) {
            dpmdthe = (ldd(io.p_metric + c + kp) - ldd(io.p_metric + c - kp)) * K.inv_2dthe;
            dpmdphi = (ldd(io.p_metric + c + dke) - ldd(io.p_metric + c + dkw)) * K.inv_2dphi;
        }
        const double rhs_v = -dpdthe * inv_rm - dpmdthe * inv_rm - (double)tr_v - tr_v_metric
                           + (double)(diffusion_v * inv_re + diffusion_v * nue_t)
                           - K.Coriolis * cor_the + K.centrifugal * ldd(&gp->cent_the);
        const double rhs_w = -dpdphi * inv_rmsinthe - dpmdphi * inv_rmsinthe - (double)tr_w - tr_w_metric
                           + (double)(diffusion_w * inv_re + diffusion_w * nue_t) - K.Coriolis * cor_phi;
        emit<MODE>(io, sp, K, ATSAT_F_U, c, rhs_u, 0.0f);
        emit<MODE>(io, sp, K, ATSAT_F_V, c, rhs_v, 0.0f);
        emit<MODE>(io, sp, K, ATSAT_F_W, c, rhs_w, 0.0f);
        if (MODE != MODE_STAGE) {
            io.aux[0][c] = rhs_u + dpdr;
            io.aux[1][c] = rhs_v + dpdthe * inv_rm;
            io.aux[2][c] = rhs_w + dpdphi * inv_rmsinthe;
        }
    }

    const float sd = K.divu_on ? (float)K.species_divu * (du.dr + 2.0f * uf * g.inv_rm + dv.dthe * g.inv_rm
                                                          + vf * g.cotanthe * g.inv_rm + dw.dphi * g.inv_rmsinthe)
                               : 0.0f;

    // ---- temperature ----
    {
        float dpstatdr = 0.0f;
        if (K.adiabatic) {
            dpstatdr = (float)((ldd(io.p_stat64 + c + P) - ldd(io.p_stat64 + c - P)) * K.inv_2dr * K.to_nd);
            const float rho_l = ldf(io.rho_mix + c);
            if (K.adiabatic_rho && rho_l > 0.0f && isfinite(rho_l)) dpstatdr *= (float)K.r_mix / rho_l;
        }
        const float pressure_t = (float)K.coeff_energy_p * (uf * ((float)dpdr + dpstatdr) + vf * (float)dpdthe * g.inv_rm
                                                             + wf * (float)dpdphi * g.inv_rmsinthe);
        D6f d;
        derivs32(io.yn32[ATSAT_F_T], dlq(ATSAT_F_T), c, P, kp, dkw, dke, KF_, d);
        const float transport_t = transport32(uf, vf, wf, d, g);
        const float diffusion_t = diffusion32(d, g);
        float radiation_t = 0.0f;
        if (K.rad_on) {
            const float rho_f = ldf(io.rho_mix + c);
            const float rho = (rho_f > 0.0f && isfinite(rho_f)) ? rho_f : (float)K.r_mix;
            if (rho > 0.0f) {
                radiation_t = (float)(K.rad_coupling * K.rad_num / K.rad_den_c) * ldf(io.q_rad + c) / rho;
                if (!isfinite(radiation_t)) radiation_t = 0.0f;
                else if (radiation_t > 0.5f) radiation_t = 0.5f;
                else if (radiation_t < -0.5f) radiation_t = -0.5f;
            }
        }
        float precip_t = 0.0f;
        if (K.precip_on) {
            precip_t = (float)(K.precip_coupling * K.precip_num * K.precip_den) * ldf(io.q_precip + c);
            if (!isfinite(precip_t)) precip_t = 0.0f;
            else if (precip_t > 0.5f) precip_t = 0.5f;
            else if (precip_t < -0.5f) precip_t = -0.5f;
        }
        float r = pressure_t - transport_t + diffusion_t * (float)K.inv_re_pr + diffusion_t * nue_t_s;
        if (K.tmf_on) r -= (float)K.tmf_chem * ldf(io.thermalmassflux + c);
        r = r + radiation_t + precip_t;
        emit<MODE>(io, sp, K, ATSAT_F_T, c, (double)r, 0.0f);
    }

    const float pc = (float)K.precip_coupling;
    const float chem = (float)K.chem;
#define ATSAT_SPECIES(FID, INV_SC_RE, EXTRA)                                                     \
    {                                                                                            \
        D6f d;                                                                                   \
        derivs32(io.yn32[FID], dlq(FID), c, P, kp, dkw, dke, KF_, d);                            \
        const float df = diffusion32(d, g);                                                      \
        float r = -transport32(uf, vf, wf, d, g) + df * (float)(INV_SC_RE) + df * nue_t_s EXTRA; \
        if (K.divu_on) r -= sd * ys(io.yn32[FID], dlq(FID), c);                                   \
        emit<MODE>(io, sp, K, FID, c, (double)r, 0.0f);                                          \
    }
    ATSAT_SPECIES(ATSAT_F_H2O, K.inv_sc_re_h2o, +pc * ldf(io.s_precip[0] + c))
    ATSAT_SPECIES(ATSAT_F_H2O_CLOUD, K.inv_sc_re_h2o, +pc * ldf(io.s_precip[1] + c))
    ATSAT_SPECIES(ATSAT_F_H2O_ICE, K.inv_sc_re_h2o, +pc * ldf(io.s_precip[2] + c))
    ATSAT_SPECIES(ATSAT_F_H2S, K.inv_sc_re_h2s, +chem * ldf(io.massflux_h2s + c))
    ATSAT_SPECIES(ATSAT_F_NH3, K.inv_sc_re_nh3, +chem * ldf(io.massflux_nh3 + c) + pc * ldf(io.s_precip[3] + c))
    ATSAT_SPECIES(ATSAT_F_NH3_CLOUD, K.inv_sc_re_nh3, +pc * ldf(io.s_precip[4] + c))
    ATSAT_SPECIES(ATSAT_F_NH3_ICE, K.inv_sc_re_nh3, +pc * ldf(io.s_precip[5] + c))
    ATSAT_SPECIES(ATSAT_F_CH4, K.inv_sc_re_ch4, +pc * ldf(io.s_precip[6] + c))
    ATSAT_SPECIES(ATSAT_F_CH4_CLOUD, K.inv_sc_re_ch4, +pc * ldf(io.s_precip[7] + c))
    ATSAT_SPECIES(ATSAT_F_CH4_ICE, K.inv_sc_re_ch4, +pc * ldf(io.s_precip[8] + c))
#undef ATSAT_SPECIES
    {
        D6f d;
        derivs32(io.yn32[ATSAT_F_NH4SH], dlq(ATSAT_F_NH4SH), c, P, kp, dkw, dke, KF_, d);
        const float df = diffusion32(d, g);
        float r = -transport32(uf, vf, wf, d, g) + ldf(io.fluxlim_nh4sh + c) + df * (float)K.inv_sc_re_nh4sh
                + df * nue_t_s + chem * ldf(io.massflux_nh4sh + c);
        if (K.divu_on) r -= sd * ys(io.yn32[ATSAT_F_NH4SH], dlq(ATSAT_F_NH4SH), c);
        emit<MODE>(io, sp, K, ATSAT_F_NH4SH, c, (double)r, 0.0f);
    }

    if (K.turb) {
        {
            D6f d;
            derivs32(io.yn32[ATSAT_F_TKE], dlq(ATSAT_F_TKE), c, P, kp, dkw, dke, KF_, d);
            const float r = -transport32(uf, vf, wf, d, g) + diffusion32(d, g) * (inv_re + nue_c * (float)K.inv_sig_k)
                          + ldf(io.tke_source + c);
            emit<MODE>(io, sp, K, ATSAT_F_TKE, c, (double)r, ldf(io.yn32[ATSAT_F_TKE] + c));
        }
        {
            D6f d;
            derivs32(io.yn32[ATSAT_F_DIS], dlq(ATSAT_F_DIS), c, P, kp, dkw, dke, KF_, d);
            const float r = -transport32(uf, vf, wf, d, g) + diffusion32(d, g) * (inv_re + nue_c * (float)K.inv_sig_w)
                          + ldf(io.dis_source + c);
            emit<MODE>(io, sp, K, ATSAT_F_DIS, c, (double)r, ldf(io.yn32[ATSAT_F_DIS] + c));
        }
    } else if (MODE == MODE_RHS || (MODE == MODE_FINAL && sp.write_all_rhs)) {
        io.rhs[ATSAT_F_TKE][c] = 0.0;
        io.rhs[ATSAT_F_DIS][c] = 0.0;
    }
}

// Prepare a drop-in step: yn32 = (float) y_n, dl_0 = (float)(live - y_n), and the FP32 copies of the
// point inputs that changed since the last step.
__global__ void __launch_bounds__(256) mixed_prepare_kernel(const KConst K, const MixedPrep pr) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    for (int q = 0; q < NPROG; q++) {
        const double yn = __ldg(pr.yn64[q] + c);
        pr.yn32[q][c] = (float)yn;
        if (pr.dl0[q]) pr.dl0[q][c] = (float)(__ldg(pr.live64[q] + c) - yn);
    }
    for (int q = 0; q < pr.nconv; q++) pr.conv_dst[q][c] = (float)__ldg(pr.conv_src[q] + c);
}

}  // namespace

cudaError_t launch_rk_stage_mixed(const KConst& kc, const MixedIO& io, const StageParams& sp, int mode,
                                  cudaStream_t s) {
    KF kf;
    kf.inv_2dr = (float)kc.inv_2dr;
    kf.inv_2dthe = (float)kc.inv_2dthe;
    kf.inv_2dphi = (float)kc.inv_2dphi;
    kf.inv_dr2 = (float)kc.inv_dr2;
    kf.inv_dthe2 = (float)kc.inv_dthe2;
    kf.inv_dphi2 = (float)kc.inv_dphi2;
    dim3 block(32, 8);
    dim3 grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    if (mode == MODE_RHS) rk_stage_mixed_kernel<MODE_RHS><<<grid, block, 0, s>>>(kc, kf, io, sp);
    else if (mode == MODE_STAGE) rk_stage_mixed_kernel<MODE_STAGE><<<grid, block, 0, s>>>(kc, kf, io, sp);
    else rk_stage_mixed_kernel<MODE_FINAL><<<grid, block, 0, s>>>(kc, kf, io, sp);
    return cudaGetLastError();
}

cudaError_t launch_mixed_prepare(const KConst& kc, const MixedPrep& pr, cudaStream_t s) {
    dim3 block(32, 8), grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    mixed_prepare_kernel<<<grid, block, 0, s>>>(kc, pr);
    return cudaGetLastError();
}

}  // namespace atsat
