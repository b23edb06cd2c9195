// Mixed-precision RK4 of the ATSAT dynamical core (RungeKuttaSat / RHSSat,
// planet/RungeKutta_Sat_Turb.cpp:110-387, planet/RHS_Sat_Turb.cpp:25-1016).
//
// GB300 executes two FP64 operations per SM per cycle against 128 FP32 ones, so the design keeps the
// per-stage work in FP32 and puts FP64 where cancellation or accumulation needs it, once per step
// where possible:
//
// * Stage inputs are FP32 increments over y_n: Y_s = y_n + dl_s, dl_s = c_in * k_{s-1}. Stencils read an
//   FP32 copy of y_n (yn32) and difference it and dl separately, so the small increment is never
//   rounded against the field. The zonal wind w carries a second FP32 word (wlo = y_n - yn32): its
//   zonal variations are tiny against |w| ~ 0.85 and would otherwise be lost in yn32's rounding.
// * The large terms of the momentum equations that cancel against each other -- the pressure and
//   p_metric gradients, the Coriolis force of the zonal jet, the w^2 cot / r metric term, the
//   centrifugal force and the buoyancy anomaly against the level mean -- depend within an RK step only
//   on p_dyn, p_metric, buoy_ref_level and y_n, which the step does not change. mixed_prepare_kernel
//   forms them in FP64 once per step and stores the balanced sums as FP32 fields ("frozen" terms).
//   Each stage adds the FP32 corrections that depend on dl (e.g. b_s - b_n = -B p_stat dl_t /
//   (t_n t_s) for the buoyancy).
// * The RK4 sums k1 + 2k2 + 2k3 + k4 are FP64 for u, v, w, t and FP32 for the 13 scalars (their
//   tendencies are FP32 quantities); the state update y_{n+1} = y_n + dt/6 * sum is FP64 for all.
#include "dyn_common.cuh"

namespace atsat {

namespace {

constexpr int NM = 4;               // u, v, w, t: FP64 accumulators

struct D6f { float dr, d2r, dthe, d2the, dphi, d2phi; };

__device__ __forceinline__ float ldf(const float* p) { return __ldg(p); }
__device__ __forceinline__ double ldd(const double* p) { return __ldg(p); }

// the six central differences of one 7-point stencil (unscaled)
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

__device__ __forceinline__ void scale6(const float* a, const MixedConstF& K, D6f& d) {
    d.dr = a[0] * K.inv_2dr;
    d.d2r = a[1] * K.inv_dr2;
    d.dthe = a[2] * K.inv_2dthe;
    d.d2the = a[3] * K.inv_dthe2;
    d.dphi = a[4] * K.inv_2dphi;
    d.d2phi = a[5] * K.inv_dphi2;
}

// derivatives of Y_s = y_n + dl (+ lo) with each part differenced on its own
__device__ __forceinline__ void derivs(const float* yn, const float* lo, const float* dl, int64_t c, int64_t P, int kp,
                                       int dkw, int dke, const MixedConstF& K, D6f& d) {
    float a[6];
    diff7(yn, c, P, kp, dkw, dke, a);
    if (lo) {
        float b[6];
        diff7(lo, c, P, kp, dkw, dke, b);
#pragma unroll
        for (int q = 0; q < 6; q++) a[q] += b[q];
    }
    if (dl) {
        float b[6];
        diff7(dl, c, P, kp, dkw, dke, b);
#pragma unroll
        for (int q = 0; q < 6; q++) a[q] += b[q];
    }
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

template <int MODE>
__device__ __forceinline__ void emit(const MixedIO& io, const StageParams& sp, const MixedConstF& K, int q,
                                     int64_t c, float r) {
    if (MODE == MODE_RHS) {
        io.rhs[q][c] = (double)r;
        return;
    }
    if (MODE == MODE_STAGE) {
        if (q < NM) {
            const double a = (sp.stage == 0) ? sp.wgt * (double)r : io.acc64[q][c] + sp.wgt * (double)r;
            io.acc64[q][c] = a;
        } else {
            const float a = (sp.stage == 0) ? (float)sp.wgt * r : io.acc32[q - NM][c] + (float)sp.wgt * r;
            io.acc32[q - NM][c] = a;
        }
        const float cr = (float)sp.c_in * r;
        float d = cr;
        if (q == ATSAT_F_TKE || q == ATSAT_F_DIS) {
            // the clamps of the stage input (RungeKutta_Sat_Turb.cpp:311-316) on Y = y_n + c_in k
            const float yn = ldf(io.yn32[q] + c);
            const float y = yn + cr;
            const float yc = (q == ATSAT_F_TKE) ? sminf(smaxf(y, 0.0f), K.tke_max) : smaxf(y, K.dis_min);
            d = yc - yn;
        }
        io.dl_out[q][c] = d;
        return;
    }
    // final stage: y_{n+1} = y_n + dt/6 (acc + k4) in FP64
    const double a = (q < NM) ? io.acc64[q][c] + sp.wgt * (double)r
                              : (double)(io.acc32[q - NM][c] + (float)sp.wgt * r);
    const double yn = ldd(io.yn64[q] + c);
    double y = yn + sp.sixth_dt * a;
    if (q == ATSAT_F_TKE) y = smin(smax(y, 0.0), K.tke_max_d);
    else if (q == ATSAT_F_DIS) y = smax(y, K.dis_min_d);
    io.out64[q][c] = y;
    if (io.out32[q]) {
        const float hi = (float)y;
        io.out32[q][c] = hi;
        if (q == ATSAT_F_W && io.wlo_out) io.wlo_out[c] = (float)(y - (double)hi);
    }
    if (sp.write_all_rhs || q < 3) io.rhs[q][c] = (double)r;
}

template <int MODE>
__global__ void __launch_bounds__(256) rk_stage_mixed_kernel(const MixedConstF K, const MixedIO io,
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
    const ColGeoF g = io.geof[(int64_t)i * K.jm + j];
    auto dl = [&](int q) -> const float* { return io.dl_in[q]; };
    auto dlv = [&](int q) -> float { return io.dl_in[q] ? ldf(io.dl_in[q] + c) : 0.0f; };

    // centre values (FP32); w and t also as y_n + increment split for the corrections
    const float dw_s = dlv(ATSAT_F_W), dt_s = dlv(ATSAT_F_T), du_s = dlv(ATSAT_F_U), dv_s = dlv(ATSAT_F_V);
    const float wn = ldf(io.yn32[ATSAT_F_W] + c) + ldf(io.wlo + c);
    const float vn = ldf(io.yn32[ATSAT_F_V] + c), un = ldf(io.yn32[ATSAT_F_U] + c);
    const float tn = ldf(io.yn32[ATSAT_F_T] + c);
    const float u = un + du_s, v = vn + dv_s, w = wn + dw_s, t = tn + dt_s;

    D6f du, dv, dw;
    derivs(io.yn32[ATSAT_F_U], nullptr, dl(ATSAT_F_U), c, P, kp, dkw, dke, K, du);
    derivs(io.yn32[ATSAT_F_V], nullptr, dl(ATSAT_F_V), c, P, kp, dkw, dke, K, dv);
    derivs(io.yn32[ATSAT_F_W], io.wlo, dl(ATSAT_F_W), c, P, kp, dkw, dke, K, dw);

    const float fz_dpr = ldf(io.fz[FZ_DPR] + c), fz_dpth = ldf(io.fz[FZ_DPTH] + c);
    const float fz_dpph = ldf(io.fz[FZ_DPPH] + c);

    const float nue_c = ldf(io.nue + c);
    const float nue_t = (K.turb_coupling != 0.0f && isfinite(nue_c)) ? K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
    const float nue_t_s = nue_t * K.inv_pr_t;

    // ---- momentum ----
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
            else buoy = K.kb * (bps / t - K.bref_scale * (float)ldd(io.buoy + i));
        }
        // stage-dependent parts of the frozen balances (terms in the increments)
        float gu_stage = 0.0f;
        if (!K.metric_split) gu_stage -= K.metric_on * (dv_s * (2.0f * vn + dv_s) + dw_s * (2.0f * wn + dw_s)) * g.inv_rm;
        if (K.cor_rad_on != 0.0f) gu_stage -= K.cor_rad_on * g.cor_rad_c * dw_s;
        const float rhs_u = ldf(io.fz[FZ_GU] + c) - fz_dpr + buoy + gu_stage - adv_u + diffusion_u * visc;
        const float rhs_v = ldf(io.fz[FZ_GV] + c) - fz_dpth - adv_v - u * v * g.inv_rm
                          + dw_s * (2.0f * wn + dw_s) * g.cotanthe * g.inv_rm - g.cor_the_c * dw_s + diffusion_v * visc;
        const float cor_phi = g.cor_phi_c * (g.costhe * (v - g.vbar0) + g.sinthe_true * (u - g.ubar0));
        const float rhs_w = ldf(io.fz[FZ_GW] + c) - fz_dpph - adv_w - (w * u + v * w * g.cotanthe) * g.inv_rm
                          + diffusion_w * visc - cor_phi;
        emit<MODE>(io, sp, K, ATSAT_F_U, c, rhs_u);
        emit<MODE>(io, sp, K, ATSAT_F_V, c, rhs_v);
        emit<MODE>(io, sp, K, ATSAT_F_W, c, rhs_w);
        if (MODE != MODE_STAGE) {
            io.aux[0][c] = (double)(rhs_u + fz_dpr);
            io.aux[1][c] = (double)(rhs_v + fz_dpth);
            io.aux[2][c] = (double)(rhs_w + fz_dpph);
        }
    }

    const float sd = K.divu_on ? K.species_divu * (du.dr + 2.0f * u * g.inv_rm + dv.dthe * g.inv_rm
                                                   + v * g.cotanthe * g.inv_rm + dw.dphi * g.inv_rmsinthe)
                               : 0.0f;

    // ---- temperature ----
    {
        const float pressure_t = K.coeff_energy_p * (u * (fz_dpr + ldf(io.fz[FZ_DPS] + c)) + v * fz_dpth + w * fz_dpph);
        D6f d;
        derivs(io.yn32[ATSAT_F_T], nullptr, dl(ATSAT_F_T), c, P, kp, dkw, dke, K, d);
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
        emit<MODE>(io, sp, K, ATSAT_F_T, c, r);
    }

    const float pc = K.precip_coupling;
    const float chem = K.chem;
#define ATSAT_SPECIES(FID, INV_SC_RE, EXTRA)                                                    \
    {                                                                                           \
        D6f d;                                                                                  \
        derivs(io.yn32[FID], nullptr, dl(FID), c, P, kp, dkw, dke, K, d);                       \
        const float df = diffusion(d, g);                                                       \
        float r = -transport(u, v, w, d, g) + df * (INV_SC_RE) + df * nue_t_s EXTRA;            \
        if (K.divu_on) r -= sd * (ldf(io.yn32[FID] + c) + dlv(FID));                             \
        emit<MODE>(io, sp, K, FID, c, r);                                                       \
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
        derivs(io.yn32[ATSAT_F_NH4SH], nullptr, dl(ATSAT_F_NH4SH), c, P, kp, dkw, dke, K, d);
        const float df = diffusion(d, g);
        float r = -transport(u, v, w, d, g) + ldf(io.fluxlim_nh4sh + c) + df * K.inv_sc_re_nh4sh + df * nue_t_s
                + chem * ldf(io.massflux_nh4sh + c);
        if (K.divu_on) r -= sd * (ldf(io.yn32[ATSAT_F_NH4SH] + c) + dlv(ATSAT_F_NH4SH));
        emit<MODE>(io, sp, K, ATSAT_F_NH4SH, c, r);
    }

    if (K.turb) {
        {
            D6f d;
            derivs(io.yn32[ATSAT_F_TKE], nullptr, dl(ATSAT_F_TKE), c, P, kp, dkw, dke, K, d);
            const float r = -transport(u, v, w, d, g) + diffusion(d, g) * (K.inv_re + nue_c * K.inv_sig_k)
                          + ldf(io.tke_source + c);
            emit<MODE>(io, sp, K, ATSAT_F_TKE, c, r);
        }
        {
            D6f d;
            derivs(io.yn32[ATSAT_F_DIS], nullptr, dl(ATSAT_F_DIS), c, P, kp, dkw, dke, K, d);
            const float r = -transport(u, v, w, d, g) + diffusion(d, g) * (K.inv_re + nue_c * K.inv_sig_w)
                          + ldf(io.dis_source + c);
            emit<MODE>(io, sp, K, ATSAT_F_DIS, c, r);
        }
    } else if (MODE == MODE_RHS || (MODE == MODE_FINAL && sp.write_all_rhs)) {
        io.rhs[ATSAT_F_TKE][c] = 0.0;
        io.rhs[ATSAT_F_DIS][c] = 0.0;
    }
}

// Once per step: the FP32 copies of y_n (and w's low word), the stage-0 increment live - y_n, the FP32
// copies of changed point inputs, and the frozen FP64 terms of the momentum equations.
__global__ void __launch_bounds__(256) mixed_prepare_kernel(const KConst K, const MixedPrep pr) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t P = K.plane;
    const int kp = K.kp;
    const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
    if (pr.write_yn32) {
        for (int q = 0; q < NPROG; q++) {
            const double yn = __ldg(pr.yn64[q] + c);
            const float hi = (float)yn;
            pr.yn32[q][c] = hi;
            if (pr.yn32_b[q]) pr.yn32_b[q][c] = hi;
            if (q == ATSAT_F_W) {
                const float lo = (float)(yn - (double)hi);
                pr.wlo[c] = lo;
                if (pr.wlo_b) pr.wlo_b[c] = lo;
            }
            if (pr.dl0[q]) pr.dl0[q][c] = (float)(__ldg(pr.live64[q] + c) - yn);
        }
    }
    for (int q = 0; q < pr.nconv; q++) pr.conv_dst[q][c] = (float)__ldg(pr.conv_src[q] + c);
    if (pr.skip_frozen) return;

    const bool interior = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    if (!interior) return;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const int64_t cw = c - k + kw, ce = c - k + ke;
    const ColGeo* g = pr.geo + ((int64_t)i * K.jm + j);
    // FP64 work is kept to the sums that cancel: every constant product comes from the host, and the
    // one reciprocal (1/t) is an FP32 estimate refined by one Newton step in FP64 (relative error
    // ~1e-14, far below what the FP32 storage of the result keeps).
    const double inv_rm = __ldg(&g->inv_rm), inv_rmsinthe = __ldg(&g->inv_rmsinthe);
    const double* p = pr.p_dyn;
    const double dpdr = (__ldg(p + c + P) - __ldg(p + c - P)) * K.inv_2dr;
    const double dpdthe = (__ldg(p + c + kp) - __ldg(p + c - kp)) * (K.inv_2dthe * inv_rm);
    const double dpdphi = (__ldg(p + ce) - __ldg(p + cw)) * (K.inv_2dphi * inv_rmsinthe);
    double dpmdthe = 0.0, dpmdphi = 0.0;
    if (K.metric_split) {
        dpmdthe = (__ldg(pr.p_metric + c + kp) - __ldg(pr.p_metric + c - kp)) * (K.inv_2dthe * inv_rm);
        dpmdphi = (__ldg(pr.p_metric + ce) - __ldg(pr.p_metric + cw)) * (K.inv_2dphi * inv_rmsinthe);
    }
    // the adiabatic term only enters rhs_t's small compression work: FP32 after the FP64 difference
    float dps = 0.0f;
    if (K.adiabatic) {
        dps = (float)(__ldg(pr.p_stat + c + P) - __ldg(pr.p_stat + c - P)) * (float)(K.inv_2dr * K.to_nd);
        const float rho_l = (float)__ldg(pr.rho_mix + c);
        if (K.adiabatic_rho && rho_l > 0.0f && isfinite(rho_l)) dps *= (float)K.r_mix / rho_l;
    }
    const double t = __ldg(pr.yn64[ATSAT_F_T] + c);
    const double ps = __ldg(pr.p_stat + c);
    // buoyancy: numerator B p (so that b = B p / t) and the anomaly at t_n
    const double bps = K.buoy_legacy ? (ps + __ldg(p + c)) * pr.bnum : ps * pr.bnum;
    double ban = 0.0;
    if (t > 0.0) {
        double r = (double)(1.0f / (float)t);
        r = r * (2.0 - t * r);
        ban = K.buoy_legacy ? bps * r : (bps * r - __ldg(pr.buoy + i));
    }
    // frozen parts of rhs_u, rhs_v, rhs_w at y_n (RHS_Sat_Turb.cpp:310-350, 388-399, 780-835)
    const double wn = __ldg(pr.yn64[ATSAT_F_W] + c);
    double gu = K.centrifugal * __ldg(&g->cent_rad);
    if (!K.metric_split) {
        const double vn = __ldg(pr.yn64[ATSAT_F_V] + c);
        gu -= K.metric_on * (vn * vn + wn * wn) * inv_rm;
    }
    if (K.cor_rad_on != 0.0) gu -= K.cor_rad_on * K.Coriolis * (__ldg(&g->cor_rad) * wn);
    // w (w cot / r) - Coriolis cor_the w, the centrifugal and the p_metric gradient
    const double gv = wn * (wn * __ldg(&g->p_pad_cot_rm) - K.Coriolis * __ldg(&g->cor_the)) - dpmdthe
                    + K.centrifugal * __ldg(&g->cent_the);
    const double gw = -dpmdphi;
    pr.fz[FZ_DPR][c] = (float)dpdr;
    pr.fz[FZ_DPTH][c] = (float)dpdthe;
    pr.fz[FZ_DPPH][c] = (float)dpdphi;
    pr.fz[FZ_DPS][c] = dps;
    pr.fz[FZ_GU][c] = (float)gu;
    pr.fz[FZ_GV][c] = (float)gv;
    pr.fz[FZ_GW][c] = (float)gw;
    pr.fz[FZ_BAN][c] = (float)ban;
    pr.fz[FZ_BPS][c] = (float)bps;
}

}  // namespace

cudaError_t launch_rk_stage_mixed(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode,
                                  cudaStream_t s) {
    dim3 block(32, 8);
    dim3 grid((kf.km + 31) / 32, (kf.jm + 7) / 8, kf.im);
    if (mode == MODE_RHS) rk_stage_mixed_kernel<MODE_RHS><<<grid, block, 0, s>>>(kf, io, sp);
    else if (mode == MODE_STAGE) rk_stage_mixed_kernel<MODE_STAGE><<<grid, block, 0, s>>>(kf, io, sp);
    else rk_stage_mixed_kernel<MODE_FINAL><<<grid, block, 0, s>>>(kf, io, sp);
    return cudaGetLastError();
}

cudaError_t launch_mixed_prepare(const KConst& kc, const MixedPrep& pr, cudaStream_t s) {
    dim3 block(32, 8), grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    mixed_prepare_kernel<<<grid, block, 0, s>>>(kc, pr);
    return cudaGetLastError();
}

}  // namespace atsat
