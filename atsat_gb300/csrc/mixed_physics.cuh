// Per-cell physics of the mixed-precision RK stage (RHSSat, planet/RHS_Sat_Turb.cpp:25-1016, with the
// stage handling of RungeKuttaSat, planet/RungeKutta_Sat_Turb.cpp:110-387), shared by the two stage
// kernels: the direct one (rk_mixed.cu, stencils read from global memory) and the TMA-tiled one
// (rk_tile.cu, stencils read from shared memory). Each kernel supplies a stencil source `Src` with
//
//   float cyn(q), cdl(q), clo()      centre values of y_n (FP32 copy), the stage increment, w's low word
//   void raw6(q, float a[6])         the six central differences of field q, every part differenced
//                                    on its own and summed (y_n, w's low word, the increment)
//
// so that both run the same arithmetic.
#pragma once

#include "dyn_common.cuh"

namespace atsat {
namespace mixed {

struct D6f { float dr, d2r, dthe, d2the, dphi, d2phi; };

__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldd(const double* p) { return __ldg(p); }

__device__ __forceinline__ void scale6(const float* a, const MixedConstF& K, D6f& d) {
    d.dr = a[0] * K.inv_2dr;
    d.d2r = a[1] * K.inv_dr2;
    d.dthe = a[2] * K.inv_2dthe;
    d.d2the = a[3] * K.inv_dthe2;
    d.dphi = a[4] * K.inv_2dphi;
    d.d2phi = a[5] * K.inv_dphi2;
}

template <class Src>
__device__ __forceinline__ void derivs(const Src& S, int q, const MixedConstF& K, D6f& d) {
    float a[6];
    S.raw6(q, a);
    scale6(a, K, d);
}

__device__ __forceinline__ float transport(float u, float v, float w, const D6f& d, const ColGeoF& g) {
    return u * d.dr + v * d.dthe * g.inv_rm + w * d.dphi * g.inv_rmsinthe;
}

__device__ __forceinline__ float diffusion(const D6f& d, const ColGeoF& g) {
    return d.d2r + d.dr * g.two_inv_rm + d.d2the * g.inv_rm2 + d.dthe * g.costhe_inv_rm2sinthe
         + d.d2phi * g.inv_rm2sinthe2;
}

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smaxf(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float sminf(float a, float b) { return (b < a) ? b : a; }

constexpr float THIRD = 0x1.555556p-2f;   // 1/3 in FP32

__device__ __forceinline__ bool is_turb(int q) { return q == ATSAT_F_TKE || q == ATSAT_F_DIS; }

// One tendency r of field q at cell c: rhs (MODE_RHS), the next stage increment (MODE_STAGE), or
// y_{n+1} (MODE_FINAL). yn_c and dl_c are the centre values of y_n (FP32) and of the stage increment.
template <int MODE>
__device__ __forceinline__ void emit(const MixedIO& io, const StageParams& sp, const MixedConstF& K, int q,
                                     int64_t c, float r, float yn_c, float dl_c) {
    if (MODE == MODE_RHS) {
        io.rhs[q][c] = f2d(r);
        return;
    }
    if (MODE == MODE_STAGE) {
        const float cr = sp.c_in_f * r;
        float d = cr;
        if (is_turb(q)) {
            // running k1 + 2 k2 + 2 k3, and the clamps of the stage input (RungeKutta_Sat_Turb.cpp:311-316)
            float* acc = io.acc_turb[q - ATSAT_F_TKE];
            acc[c] = (sp.stage == 0) ? sp.wgt_f * r : acc[c] + sp.wgt_f * r;
            const float y = yn_c + cr;
            const float yc = (q == ATSAT_F_TKE) ? sminf(smaxf(y, 0.0f), K.tke_max) : smaxf(y, K.dis_min);
            d = yc - yn_c;
        }
        io.dl_out[q][c] = d;
        return;
    }
    // y_{n+1} = y_n + increment: the increment in FP32, the sum in FP64
    float inc;
    if (is_turb(q)) inc = sp.sixth_dt_f * (io.acc_turb[q - ATSAT_F_TKE][c] + r);
    else inc = THIRD * (ldf(io.dl1[q] + c) + 2.0f * ldf(io.dl2[q] + c) + dl_c) + sp.sixth_dt_f * r;
    double y = ldd(io.yn64[q] + c) + f2d(inc);
    if (q == ATSAT_F_TKE) y = smin(smax(y, 0.0), K.tke_max_d);
    else if (q == ATSAT_F_DIS) y = smax(y, K.dis_min_d);
    io.out64[q][c] = y;
    if (io.out32[q]) {
        const float hi = d2f(y);
        io.out32[q][c] = hi;
        if (q == ATSAT_F_W && io.wlo_out) io.wlo_out[c] = d2f(y - f2d(hi));
    }
    if (sp.write_all_rhs || q < 3) io.rhs[q][c] = f2d(r);
}

// what the scalar equations take from the momentum / temperature part of a cell
struct CellState {
    float u, v, w;          // stage velocities
    float sd;               // species_divu * div u (0 when off)
    float nue_c;            // eddy viscosity as stored
    float nue_t_s;          // nue_t / Pr_t
};

// The tracers' view of a cell without the momentum part (species_divu off): stage velocities from the
// centre values and the eddy viscosity terms, exactly as momentum_t forms them.
template <class Src>
__device__ __forceinline__ CellState tracer_state(const MixedConstF& K, const MixedIO& io, const Src& S, int64_t c) {
    const float u = S.cyn(ATSAT_F_U) + S.cdl(ATSAT_F_U);
    const float v = S.cyn(ATSAT_F_V) + S.cdl(ATSAT_F_V);
    const float w = (S.cyn(ATSAT_F_W) + S.clo()) + S.cdl(ATSAT_F_W);
    const float nue_c = ldf(io.nue + c);
    const float nue_t = (K.turb_coupling != 0.0f && isfinite(nue_c)) ? K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
    return CellState{u, v, w, 0.0f, nue_c, nue_t * K.inv_pr_t};
}

// rhs_u, rhs_v, rhs_w (RHS_Sat_Turb.cpp:300-440) and rhs_t (:460-560) of one cell, emitted.
template <int MODE, class Src>
__device__ __forceinline__ CellState momentum_t(const MixedConstF& K, const MixedIO& io, const StageParams& sp,
                                                const Src& S, int i, int64_t c, const ColGeoF& g) {
    const float dw_s = S.cdl(ATSAT_F_W), dt_s = S.cdl(ATSAT_F_T);
    const float du_s = S.cdl(ATSAT_F_U), dv_s = S.cdl(ATSAT_F_V);
    const float un = S.cyn(ATSAT_F_U), vn = S.cyn(ATSAT_F_V);
    const float wn = S.cyn(ATSAT_F_W) + S.clo(), tn = S.cyn(ATSAT_F_T);
    const float u = un + du_s, v = vn + dv_s, w = wn + dw_s, t = tn + dt_s;

    D6f du, dv, dw;
    derivs(S, ATSAT_F_U, K, du);
    derivs(S, ATSAT_F_V, K, dv);
    derivs(S, ATSAT_F_W, K, dw);

    const float fz_dpr = ldf(io.fz[FZ_DPR] + c), fz_dpth = ldf(io.fz[FZ_DPTH] + c);
    const float fz_dpph = ldf(io.fz[FZ_DPPH] + c);

    const float nue_c = ldf(io.nue + c);
    const float nue_t = (K.turb_coupling != 0.0f && isfinite(nue_c)) ? K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
    const float nue_t_s = nue_t * K.inv_pr_t;

    {
        const float adv_u = u * du.dr + v * du.dthe * g.inv_rm + w * du.dphi * g.inv_rmsinthe;
        const float adv_v = u * dv.dr + v * dv.dthe * g.inv_rm + w * dv.dphi * g.inv_rmsinthe;
        const float adv_w = u * dw.dr + v * dw.dthe * g.inv_rm + w * dw.dphi * g.inv_rmsinthe;
        const float diffusion_u = du.d2r + 2.0f * u * g.inv_rm2 + du.d2the * g.inv_rm2 + 4.0f * du.dr * g.inv_rm
                                + du.dthe * g.costhe_inv_rm2sinthe + du.d2phi * g.inv_rm2sinthe2;
        const float diffusion_v = dv.d2r + dv.dr * g.two_inv_rm + dv.d2the * g.inv_rm2
                                + dv.dthe * g.costhe_inv_rm2sinthe - g.v_metric * v
                                + dv.d2phi * g.inv_rm2sinthe2 + 2.0f * du.dthe * g.inv_rm2
                                - dw.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
        const float diffusion_w = dw.d2r + dw.dr * g.two_inv_rm + dw.d2the * g.inv_rm2
                                + dw.dthe * g.costhe_inv_rm2sinthe - g.v_metric * w
                                + dw.d2phi * g.inv_rm2sinthe2 + 2.0f * du.dphi * g.inv_rm2sinthe
                                + dv.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
        const float visc = K.inv_re + nue_t;

        // buoyancy at the stage temperature: the frozen FP64 anomaly at t_n plus the FP32 change
        float buoy = 0.0f;
        if (t > 0.0f && !K.hydro_buoy) {
            const float bps = ldf(io.fz[FZ_BPS] + c);
            if (tn > 0.0f) buoy = K.kb * (ldf(io.fz[FZ_BAN] + c) - bps * dt_s / (tn * t));
            else buoy = K.kb * (bps / t - K.bref_scale * d2f(ldd(io.buoy + i)));
        }
        // stage-dependent parts of the frozen balances (terms in the increments)
        float gu_stage = 0.0f;
        if (!K.metric_split) gu_stage += K.metric_on * (dv_s * (2.0f * vn + dv_s) + dw_s * (2.0f * wn + dw_s)) * g.inv_rm;
        if (K.cor_rad_on != 0.0f) gu_stage -= K.cor_rad_on * g.cor_rad_c * dw_s;
        const float rhs_u = ldf(io.fz[FZ_GU] + c) - fz_dpr + buoy + gu_stage - adv_u + diffusion_u * visc;
        const float rhs_v = ldf(io.fz[FZ_GV] + c) - fz_dpth - adv_v - u * v * g.inv_rm
                          + dw_s * (2.0f * wn + dw_s) * g.cotanthe * g.inv_rm - g.cor_the_c * dw_s + diffusion_v * visc;
        const float cor_phi = g.cor_phi_c * (g.costhe * (v - g.vbar0) + g.sinthe_true * (u - g.ubar0));
        const float rhs_w = ldf(io.fz[FZ_GW] + c) - fz_dpph - adv_w - (w * u + v * w * g.cotanthe) * g.inv_rm
                          + diffusion_w * visc - cor_phi;
        emit<MODE>(io, sp, K, ATSAT_F_U, c, rhs_u, un, du_s);
        emit<MODE>(io, sp, K, ATSAT_F_V, c, rhs_v, vn, dv_s);
        emit<MODE>(io, sp, K, ATSAT_F_W, c, rhs_w, S.cyn(ATSAT_F_W), dw_s);
        if (MODE != MODE_STAGE) {
            io.aux[0][c] = f2d(rhs_u + fz_dpr);
            io.aux[1][c] = f2d(rhs_v + fz_dpth);
            io.aux[2][c] = f2d(rhs_w + fz_dpph);
        }
    }

    const float sd = K.divu_on ? K.species_divu * (du.dr + 2.0f * u * g.inv_rm + dv.dthe * g.inv_rm
                                                   + v * g.cotanthe * g.inv_rm + dw.dphi * g.inv_rmsinthe)
                               : 0.0f;

    {
        const float pressure_t = K.coeff_energy_p * (u * (fz_dpr + ldf(io.fz[FZ_DPS] + c)) + v * fz_dpth + w * fz_dpph);
        D6f d;
        derivs(S, ATSAT_F_T, K, d);
        float radiation_t = 0.0f;
        if (K.rad_on) {
            const float rho_f = ldf(io.rho_mix + c);
            const float rho = (rho_f > 0.0f && isfinite(rho_f)) ? rho_f : K.r_mix;
            if (rho > 0.0f) {
                radiation_t = K.rad_factor * ldf(io.q_rad + c) / rho;
                if (!isfinite(radiation_t)) radiation_t = 0.0f;
                else if (radiation_t > 0.5f) radiation_t = 0.5f;
                else if (radiation_t < -0.5f) radiation_t = -0.5f;
            }
        }
        float precip_t = 0.0f;
        if (K.precip_on) {
            precip_t = K.precip_factor * ldf(io.q_precip + c);
            if (!isfinite(precip_t)) precip_t = 0.0f;
            else if (precip_t > 0.5f) precip_t = 0.5f;
            else if (precip_t < -0.5f) precip_t = -0.5f;
        }
        const float diffusion_t = diffusion(d, g);
        float r = pressure_t - transport(u, v, w, d, g) + diffusion_t * K.inv_re_pr + diffusion_t * nue_t_s;
        if (K.tmf_on) r -= K.tmf_chem * ldf(io.thermalmassflux + c);
        r = r + radiation_t + precip_t;
        emit<MODE>(io, sp, K, ATSAT_F_T, c, r, tn, dt_s);
    }
    return CellState{u, v, w, sd, nue_c, nue_t_s};
}

// the tracer equations (RHS_Sat_Turb.cpp:580-1000): q = 4 .. 16, q a compile-time constant after
// unrolling; tke and dis only when turbulence is on.
template <int MODE, class Src>
__device__ __forceinline__ void scalar(int q, const MixedConstF& K, const MixedIO& io, const StageParams& sp,
                                       const Src& S, int64_t c, const ColGeoF& g, const CellState& cs) {
    D6f d;
    derivs(S, q, K, d);
    const float df = diffusion(d, g);
    const float yn_c = S.cyn(q), dl_c = S.cdl(q);
    float r;
    if (q == ATSAT_F_TKE || q == ATSAT_F_DIS) {
        const float inv_sig = (q == ATSAT_F_TKE) ? K.inv_sig_k : K.inv_sig_w;
        const float* src = (q == ATSAT_F_TKE) ? io.tke_source : io.dis_source;
        r = -transport(cs.u, cs.v, cs.w, d, g) + df * (K.inv_re + cs.nue_c * inv_sig) + ldf(src + c);
    } else if (q == ATSAT_F_NH4SH) {
        r = -transport(cs.u, cs.v, cs.w, d, g) + ldf(io.fluxlim_nh4sh + c) + df * K.inv_sc_re_nh4sh
          + df * cs.nue_t_s + K.chem * ldf(io.massflux_nh4sh + c);
        if (K.divu_on) r -= cs.sd * (yn_c + dl_c);
    } else {
        float inv_sc_re, extra;
        const float pc = K.precip_coupling;
        switch (q) {
            case ATSAT_F_H2O: inv_sc_re = K.inv_sc_re_h2o; extra = pc * ldf(io.s_precip[0] + c); break;
            case ATSAT_F_H2O_CLOUD: inv_sc_re = K.inv_sc_re_h2o; extra = pc * ldf(io.s_precip[1] + c); break;
            case ATSAT_F_H2O_ICE: inv_sc_re = K.inv_sc_re_h2o; extra = pc * ldf(io.s_precip[2] + c); break;
            case ATSAT_F_H2S: inv_sc_re = K.inv_sc_re_h2s; extra = K.chem * ldf(io.massflux_h2s + c); break;
            case ATSAT_F_NH3:
                inv_sc_re = K.inv_sc_re_nh3;
                extra = K.chem * ldf(io.massflux_nh3 + c) + pc * ldf(io.s_precip[3] + c);
                break;
            case ATSAT_F_NH3_CLOUD: inv_sc_re = K.inv_sc_re_nh3; extra = pc * ldf(io.s_precip[4] + c); break;
            case ATSAT_F_NH3_ICE: inv_sc_re = K.inv_sc_re_nh3; extra = pc * ldf(io.s_precip[5] + c); break;
            case ATSAT_F_CH4: inv_sc_re = K.inv_sc_re_ch4; extra = pc * ldf(io.s_precip[6] + c); break;
            case ATSAT_F_CH4_CLOUD: inv_sc_re = K.inv_sc_re_ch4; extra = pc * ldf(io.s_precip[7] + c); break;
            default: inv_sc_re = K.inv_sc_re_ch4; extra = pc * ldf(io.s_precip[8] + c); break;
        }
        r = -transport(cs.u, cs.v, cs.w, d, g) + df * inv_sc_re + df * cs.nue_t_s + extra;
        if (K.divu_on) r -= cs.sd * (yn_c + dl_c);
    }
    emit<MODE>(io, sp, K, q, c, r, yn_c, dl_c);
}

}  // namespace mixed
}  // namespace atsat
