// TMA-tiled RK stage of the momentum and temperature equations (rhs_u, rhs_v, rhs_w, rhs_t:
// RHS_Sat_Turb.cpp:300-560 with the stage handling of RungeKutta_Sat_Turb.cpp:250-375), the partner of
// the tracer kernel in rk_tracer_tile.cu (species_divu off). Same arithmetic as mixed_physics.cuh's
// momentum_t, term by term.
//
// A block owns 32 x 8 x 2 cells (k, j, i). A producer warp streams, in the consumers' order, nue; the
// halo boxes (40 x 10 x 4 floats) of u, v, w (with w's low word) and t, each field's y_n copy then its
// stage increment; and point boxes (32 x 8 x 2 floats) of the frozen FP64-formed terms and the
// temperature's inputs, a few at a time: {DPR, GU, BAN, BPS} for rhs_u, {DPTH, GV} for rhs_v,
// {DPPH, GW} for rhs_w, {DPS, rho_mix, Q_rad, Q_precip, thermalmassflux} for rhs_t. The derivatives of
// u and v stay in registers until w's boxes arrive; no more than three halo boxes are held at once.
// The kernel is issue-latency bound (~700 instructions per cell), so it is held to 72 registers for three
// blocks (27 warps) per SM: 1.4x faster than two blocks at 84-96 registers. Deeper rings (every item of
// a tile in flight) gain nothing.
#include <cuda.h>

#include "mixed_physics.cuh"
#include "tma_pipe.cuh"

namespace atsat {

namespace {

using namespace mixed;
using namespace tma;

constexpr int TI = TILE_I;                                // 2 radial levels per thread
constexpr int PL = TILE_BX * TILE_BY;                     // 400
constexpr int BOX_F = PL * TILE_BZ;                       // 1600
constexpr int SEAM_F = TILE_SEAM_X * TILE_J * TI;         // 64
constexpr int HSLOT_F = BOX_F + SEAM_F;                   // 1664 floats = 6656 bytes
constexpr int PSLOT_F = TILE_K * TILE_J * TI;             // 512 floats = 2048 bytes
constexpr uint32_t BOX_BYTES = BOX_F * 4, SEAM_BYTES = SEAM_F * 4, PT_BYTES = PSLOT_F * 4;
constexpr int NHS = 5, NPS = 8;
constexpr int NCW = TILE_J;
constexpr int THREADS = (NCW + 1) * 32;
constexpr int GEO_F = TI * TILE_J * 16;
constexpr size_t SMEM_BYTES = (size_t)NHS * HSLOT_F * 4 + (size_t)NPS * PSLOT_F * 4 + (size_t)GEO_F * 4
                            + 2 * (NHS + NPS) * 8;

static_assert((HSLOT_F * 4) % 128 == 0 && (PSLOT_F * 4) % 128 == 0 && (BOX_F * 4) % 128 == 0, "slot alignment");

template <int NS>
__device__ __forceinline__ bool wait_items(const Ring& rg, int n0, int n1, long long limit) {
    bool ok = true;
#pragma unroll
    for (int n = n0; n < n1; n++) ok = ok && mbar_wait(rg.full(n % NS), (uint32_t)((n / NS) & 1), limit);
    return !__any_sync(0xffffffffu, !ok);
}

__device__ __forceinline__ void d7(const float* s, int o, int ow, int oe, float* e) {
    const float x = s[o];
    const float rp = s[o + PL], rn = s[o - PL];
    const float tp = s[o + TILE_BX], tn = s[o - TILE_BX];
    const float pe = s[oe], pw = s[ow];
    e[0] = rp - rn;
    e[1] = rp - 2.0f * x + rn;
    e[2] = tp - tn;
    e[3] = tp - 2.0f * x + tn;
    e[4] = pe - pw;
    e[5] = pe - 2.0f * x + pw;
}

// point items (after nue, the first item): rhs_u group, rhs_v group, rhs_w group, rhs_t group
enum { P_NUE = 0, P_DPR = 1, P_GU, P_BAN, P_BPS, P_DPTH, P_GV, P_DPPH, P_GW, P_DPS, P_RHO, P_QRAD, P_QPRECIP, P_TMF,
       N_PT = 14 };

template <int MODE, bool HAS_DL>
__global__ void __launch_bounds__(THREADS, 3)
rk_mom_tile_kernel(const __grid_constant__ CUtensorMap map_main, const __grid_constant__ CUtensorMap map_seam,
                   const __grid_constant__ CUtensorMap map_pt, const MixedConstF K, const MixedIO io,
                   const StageParams sp, const TracerPlan plan) {
    extern __shared__ __align__(128) float smem[];
    float* hs = smem;
    float* ps = hs + NHS * HSLOT_F;
    float* sgeo = ps + NPS * PSLOT_F;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sgeo + GEO_F);
    const Ring rh{smem_u32(bars), smem_u32(bars + NHS)};
    const Ring rp{smem_u32(bars + 2 * NHS), smem_u32(bars + 2 * NHS + NPS)};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int k0 = blockIdx.x * TILE_K;
    const int j0 = 2 + blockIdx.y * TILE_J;
    const int i0 = 1 + blockIdx.z * TI;
    int seam = 0, xs = 0;
    if (k0 == 0 && K.km - 2 > k0 + TILE_K + 3) { seam = 1; xs = (K.km - 2) & ~3; }
    else if (k0 > 0 && K.km - 2 >= k0 && K.km - 2 < k0 + TILE_K) { seam = 2; xs = 0; }

    if (smem_u32(smem) & 127u) {
        if (threadIdx.x == 0) atomicOr(plan.err, ERR_ALIGN);
        return;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NHS; s++) { mbar_init(rh.full(s), 1); mbar_init(rh.empty(s), NCW); }
        for (int s = 0; s < NPS; s++) { mbar_init(rp.full(s), 1); mbar_init(rp.empty(s), NCW); }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        if (lane == 0) {
            int nh = 0, np = 0;
            bool ok = true;
            const int n_issue = plan.n_items - plan.withhold;
            for (int n = 0; n < n_issue && ok; n++) {
                if (plan.kind[n] == 0) {
                    const int s = nh % NHS;
                    if (nh >= NHS && !mbar_wait(rh.empty(s), (uint32_t)(((nh / NHS) - 1) & 1), plan.wait_limit)) {
                        ok = false;
                        break;
                    }
                    const uint32_t dst = smem_u32(hs + s * HSLOT_F);
                    mbar_expect_tx(rh.full(s), BOX_BYTES + (seam ? SEAM_BYTES : 0u));
                    tma_load_4d(dst, &map_main, k0 - 4, j0 - 1, i0 - 1, plan.arr[n], rh.full(s));
                    if (seam) tma_load_4d(dst + BOX_BYTES, &map_seam, xs, j0, i0, plan.arr[n], rh.full(s));
                    nh++;
                } else {
                    const int s = np % NPS;
                    if (np >= NPS && !mbar_wait(rp.empty(s), (uint32_t)(((np / NPS) - 1) & 1), plan.wait_limit)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(rp.full(s), PT_BYTES);
                    tma_load_4d(smem_u32(ps + s * PSLOT_F), &map_pt, k0, j0, i0, plan.arr[n], rp.full(s));
                    np++;
                }
            }
            if (!ok) atomicOr(plan.err, ERR_PRODUCER);
            for (int m = (nh > NHS ? nh - NHS : 0); m < nh; m++)
                if (!mbar_wait(rh.full(m % NHS), (uint32_t)((m / NHS) & 1))) break;
            for (int m = (np > NPS ? np - NPS : 0); m < np; m++)
                if (!mbar_wait(rp.full(m % NPS), (uint32_t)((m / NPS) & 1))) break;
        }
        return;
    }

    const int j = j0 + warp, k = k0 + lane;
    {
        const int ii = lane >> 4, f = lane & 15;
        const int i = i0 + ii;
        float v = 0.0f;
        if (i < K.im && j < K.jm) v = __ldg(reinterpret_cast<const float*>(io.geof + ((int64_t)i * K.jm + j)) + f);
        sgeo[(ii * TILE_J + warp) * 16 + f] = v;
        __syncwarp();
    }
    bool valid[TI];
    int64_t c[TI];
    int o[TI], ow[TI], oe[TI], pidx[TI];
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        const int i = i0 + ii;
        valid[ii] = (k <= K.km - 2) && (j <= K.jm - 3) && (i <= K.im - 2);
        c[ii] = ((int64_t)i * K.jm + j) * K.kp + k;
        const int row = (1 + ii) * PL + (warp + 1) * TILE_BX;
        o[ii] = row + lane + 4;
        ow[ii] = o[ii] - 1;
        oe[ii] = o[ii] + 1;
        if (k == 0)
            ow[ii] = (seam == 1) ? BOX_F + (ii * TILE_J + warp) * TILE_SEAM_X + ((K.km - 2) - xs)
                                 : row + (K.km - 2) - (k0 - 4);
        if (k == K.km - 2)
            oe[ii] = (seam == 2) ? BOX_F + (ii * TILE_J + warp) * TILE_SEAM_X + (0 - xs) : row + 0 - (k0 - 4);
        pidx[ii] = (ii * TILE_J + warp) * TILE_K + lane;
    }
    auto fail = [&]() { if (lane == 0) atomicOr(plan.err, ERR_CONSUMER); };
    auto P = [&](int n) -> const float* { return ps + (n % NPS) * PSLOT_F; };
    auto H = [&](int n) -> const float* { return hs + (n % NHS) * HSLOT_F; };
    auto G = [&](int ii) -> const ColGeoF& { return *reinterpret_cast<const ColGeoF*>(sgeo + (ii * TILE_J + warp) * 16); };

    // nue -> eddy viscosity terms
    float nue_t[TI], nue_t_s[TI];
    if (!wait_items<NPS>(rp, P_NUE, P_NUE + 1, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        const float nue_c = P(P_NUE)[pidx[ii]];
        nue_t[ii] = (K.turb_coupling != 0.0f && isfinite(nue_c)) ? K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
        nue_t_s[ii] = nue_t[ii] * K.inv_pr_t;
    }
    slot_reads_done();
    release<NPS>(rp, P_NUE, P_NUE + 1);

    // halo items: u_yn [u_dl] | v_yn [v_dl] | w_yn w_lo [w_dl] | t_yn [t_dl]
    constexpr int DL = HAS_DL ? 1 : 0;
    constexpr int hU = 0, hV = 1 + DL, hW = 2 + 2 * DL, hT = 4 + 3 * DL, hEnd = 5 + 4 * DL;
    float un[TI], du_s[TI], vn[TI], dv_s[TI], wn[TI], dw_s[TI], wyn[TI];
    D6f du[TI], dv[TI];
    // u
    if (!wait_items<NHS>(rh, hU, hV, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        float a[6];
        d7(H(hU), o[ii], ow[ii], oe[ii], a);
        if (HAS_DL) {
            float b[6];
            d7(H(hU + 1), o[ii], ow[ii], oe[ii], b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
        scale6(a, K, du[ii]);
        un[ii] = H(hU)[o[ii]];
        du_s[ii] = HAS_DL ? H(hU + 1)[o[ii]] : 0.0f;
    }
    slot_reads_done();
    release<NHS>(rh, hU, hV);
    // v
    if (!wait_items<NHS>(rh, hV, hW, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        float a[6];
        d7(H(hV), o[ii], ow[ii], oe[ii], a);
        if (HAS_DL) {
            float b[6];
            d7(H(hV + 1), o[ii], ow[ii], oe[ii], b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
        scale6(a, K, dv[ii]);
        vn[ii] = H(hV)[o[ii]];
        dv_s[ii] = HAS_DL ? H(hV + 1)[o[ii]] : 0.0f;
    }
    slot_reads_done();
    release<NHS>(rh, hV, hW);
    // w (y_n, low word, increment) and the momentum equations' transport and viscous parts
    float adv_u[TI], adv_v[TI], adv_w[TI], dif_u[TI], dif_v[TI], dif_w[TI];
    if (!wait_items<NHS>(rh, hW, hT, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        float a[6], b[6];
        d7(H(hW), o[ii], ow[ii], oe[ii], a);
        d7(H(hW + 1), o[ii], ow[ii], oe[ii], b);
#pragma unroll
        for (int r = 0; r < 6; r++) a[r] += b[r];
        if (HAS_DL) {
            d7(H(hW + 2), o[ii], ow[ii], oe[ii], b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
        D6f dw;
        scale6(a, K, dw);
        wyn[ii] = H(hW)[o[ii]];
        wn[ii] = wyn[ii] + H(hW + 1)[o[ii]];
        dw_s[ii] = HAS_DL ? H(hW + 2)[o[ii]] : 0.0f;
        const ColGeoF& g = G(ii);
        const float u = un[ii] + du_s[ii], v = vn[ii] + dv_s[ii], w = wn[ii] + dw_s[ii];
        const D6f& Du = du[ii];
        const D6f& Dv = dv[ii];
        adv_u[ii] = u * Du.dr + v * Du.dthe * g.inv_rm + w * Du.dphi * g.inv_rmsinthe;
        adv_v[ii] = u * Dv.dr + v * Dv.dthe * g.inv_rm + w * Dv.dphi * g.inv_rmsinthe;
        adv_w[ii] = u * dw.dr + v * dw.dthe * g.inv_rm + w * dw.dphi * g.inv_rmsinthe;
        dif_u[ii] = Du.d2r + 2.0f * u * g.inv_rm2 + Du.d2the * g.inv_rm2 + 4.0f * Du.dr * g.inv_rm
                  + Du.dthe * g.costhe_inv_rm2sinthe + Du.d2phi * g.inv_rm2sinthe2;
        dif_v[ii] = Dv.d2r + Dv.dr * g.two_inv_rm + Dv.d2the * g.inv_rm2
                  + Dv.dthe * g.costhe_inv_rm2sinthe - g.v_metric * v
                  + Dv.d2phi * g.inv_rm2sinthe2 + 2.0f * Du.dthe * g.inv_rm2
                  - dw.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
        dif_w[ii] = dw.d2r + dw.dr * g.two_inv_rm + dw.d2the * g.inv_rm2
                  + dw.dthe * g.costhe_inv_rm2sinthe - g.v_metric * w
                  + dw.d2phi * g.inv_rm2sinthe2 + 2.0f * Du.dphi * g.inv_rm2sinthe
                  + Dv.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
    }
    slot_reads_done();
    release<NHS>(rh, hW, hT);

    float dpr[TI], dpth[TI], dpph[TI];
    // rhs_u: frozen GU, DPR, the buoyancy anomaly BAN, BPS; needs the stage temperature -> t's centre values
    // come with t's halo items below, so u waits for them
    if (!wait_items<NHS>(rh, hT, hEnd, plan.wait_limit)) { fail(); return; }
    float tn[TI], dt_s[TI];
    D6f dtd[TI];
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        float a[6];
        d7(H(hT), o[ii], ow[ii], oe[ii], a);
        if (HAS_DL) {
            float b[6];
            d7(H(hT + 1), o[ii], ow[ii], oe[ii], b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
        scale6(a, K, dtd[ii]);
        tn[ii] = H(hT)[o[ii]];
        dt_s[ii] = HAS_DL ? H(hT + 1)[o[ii]] : 0.0f;
    }
    slot_reads_done();
    release<NHS>(rh, hT, hEnd);

    if (!wait_items<NPS>(rp, P_DPR, P_DPTH, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        if (!valid[ii]) continue;
        const ColGeoF& g = G(ii);
        const int x = pidx[ii];
        const float t = tn[ii] + dt_s[ii];
        dpr[ii] = P(P_DPR)[x];
        float buoy = 0.0f;
        if (t > 0.0f && !K.hydro_buoy) {
            const float bps = P(P_BPS)[x];
            if (tn[ii] > 0.0f) buoy = K.kb * (P(P_BAN)[x] - bps * dt_s[ii] / (tn[ii] * t));
            else buoy = K.kb * (bps / t - K.bref_scale * d2f(ldd(io.buoy + i0 + ii)));
        }
        float gu_stage = 0.0f;
        if (!K.metric_split)
            gu_stage += K.metric_on * (dv_s[ii] * (2.0f * vn[ii] + dv_s[ii]) + dw_s[ii] * (2.0f * wn[ii] + dw_s[ii])) * g.inv_rm;
        if (K.cor_rad_on != 0.0f) gu_stage -= K.cor_rad_on * g.cor_rad_c * dw_s[ii];
        const float visc = K.inv_re + nue_t[ii];
        const float rhs_u = P(P_GU)[x] - dpr[ii] + buoy + gu_stage - adv_u[ii] + dif_u[ii] * visc;
        emit<MODE>(io, sp, K, ATSAT_F_U, c[ii], rhs_u, un[ii], du_s[ii]);
        if (MODE != MODE_STAGE) io.aux[0][c[ii]] = f2d(rhs_u + dpr[ii]);
    }
    release<NPS>(rp, P_DPR, P_DPTH);

    if (!wait_items<NPS>(rp, P_DPTH, P_DPPH, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        if (!valid[ii]) continue;
        const ColGeoF& g = G(ii);
        const int x = pidx[ii];
        const float u = un[ii] + du_s[ii], v = vn[ii] + dv_s[ii];
        dpth[ii] = P(P_DPTH)[x];
        const float visc = K.inv_re + nue_t[ii];
        const float rhs_v = P(P_GV)[x] - dpth[ii] - adv_v[ii] - u * v * g.inv_rm
                          + dw_s[ii] * (2.0f * wn[ii] + dw_s[ii]) * g.cotanthe * g.inv_rm - g.cor_the_c * dw_s[ii]
                          + dif_v[ii] * visc;
        emit<MODE>(io, sp, K, ATSAT_F_V, c[ii], rhs_v, vn[ii], dv_s[ii]);
        if (MODE != MODE_STAGE) io.aux[1][c[ii]] = f2d(rhs_v + dpth[ii]);
    }
    release<NPS>(rp, P_DPTH, P_DPPH);

    if (!wait_items<NPS>(rp, P_DPPH, P_DPS, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        if (!valid[ii]) continue;
        const ColGeoF& g = G(ii);
        const int x = pidx[ii];
        const float u = un[ii] + du_s[ii], v = vn[ii] + dv_s[ii], w = wn[ii] + dw_s[ii];
        dpph[ii] = P(P_DPPH)[x];
        const float visc = K.inv_re + nue_t[ii];
        const float cor_phi = g.cor_phi_c * (g.costhe * (v - g.vbar0) + g.sinthe_true * (u - g.ubar0));
        const float rhs_w = P(P_GW)[x] - dpph[ii] - adv_w[ii] - (w * u + v * w * g.cotanthe) * g.inv_rm
                          + dif_w[ii] * visc - cor_phi;
        emit<MODE>(io, sp, K, ATSAT_F_W, c[ii], rhs_w, wyn[ii], dw_s[ii]);
        if (MODE != MODE_STAGE) io.aux[2][c[ii]] = f2d(rhs_w + dpph[ii]);
    }
    release<NPS>(rp, P_DPPH, P_DPS);

    // rhs_t (RHS_Sat_Turb.cpp:460-560)
    if (!wait_items<NPS>(rp, P_DPS, N_PT, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        if (!valid[ii]) continue;
        const ColGeoF& g = G(ii);
        const int x = pidx[ii];
        const float u = un[ii] + du_s[ii], v = vn[ii] + dv_s[ii], w = wn[ii] + dw_s[ii];
        const float pressure_t = K.coeff_energy_p * (u * (dpr[ii] + P(P_DPS)[x]) + v * dpth[ii] + w * dpph[ii]);
        float radiation_t = 0.0f;
        if (K.rad_on) {
            const float rho_f = P(P_RHO)[x];
            const float rho = (rho_f > 0.0f && isfinite(rho_f)) ? rho_f : K.r_mix;
            if (rho > 0.0f) {
                radiation_t = K.rad_factor * P(P_QRAD)[x] / rho;
                if (!isfinite(radiation_t)) radiation_t = 0.0f;
                else if (radiation_t > 0.5f) radiation_t = 0.5f;
                else if (radiation_t < -0.5f) radiation_t = -0.5f;
            }
        }
        float precip_t = 0.0f;
        if (K.precip_on) {
            precip_t = K.precip_factor * P(P_QPRECIP)[x];
            if (!isfinite(precip_t)) precip_t = 0.0f;
            else if (precip_t > 0.5f) precip_t = 0.5f;
            else if (precip_t < -0.5f) precip_t = -0.5f;
        }
        const D6f& d = dtd[ii];
        const float diffusion_t = diffusion(d, g);
        float r = pressure_t - transport(u, v, w, d, g) + diffusion_t * K.inv_re_pr + diffusion_t * nue_t_s[ii];
        if (K.tmf_on) r -= K.tmf_chem * P(P_TMF)[x];
        r = r + radiation_t + precip_t;
        emit<MODE>(io, sp, K, ATSAT_F_T, c[ii], r, tn[ii], dt_s[ii]);
    }
    release<NPS>(rp, P_DPS, N_PT);
}

template <int MODE, bool HAS_DL>
cudaError_t launch_one(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                       const TracerPlan& plan, dim3 grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(rk_mom_tile_kernel<MODE, HAS_DL>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    rk_mom_tile_kernel<MODE, HAS_DL><<<grid, THREADS, SMEM_BYTES, s>>>(
        *reinterpret_cast<const CUtensorMap*>(maps.main), *reinterpret_cast<const CUtensorMap*>(maps.seam),
        *reinterpret_cast<const CUtensorMap*>(maps.pt2), kf, io, sp, plan);
    return cudaGetLastError();
}

}  // namespace

int mom_plan_items(bool has_dl) { return N_PT + (has_dl ? 9 : 5); }

cudaError_t launch_rk_mom_tile(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                               const TracerPlan& plan, int mode, cudaStream_t s) {
    const int nk = (kf.km - 1 + TILE_K - 1) / TILE_K;
    const int nj = (kf.jm - 4 + TILE_J - 1) / TILE_J;
    const int ni = (kf.im - 2 + TI - 1) / TI;
    if (nk <= 0 || nj <= 0 || ni <= 0) return cudaSuccess;
    if (mode == MODE_RHS || kf.divu_on || plan.n_items > TRACER_MAX_ITEMS) return cudaErrorInvalidValue;
    const dim3 grid(nk, nj, ni);
    const bool has_dl = io.dl_in[0] != nullptr;
    if (mode == MODE_STAGE)
        return has_dl ? launch_one<MODE_STAGE, true>(maps, kf, io, sp, plan, grid, s)
                      : launch_one<MODE_STAGE, false>(maps, kf, io, sp, plan, grid, s);
    return has_dl ? launch_one<MODE_FINAL, true>(maps, kf, io, sp, plan, grid, s)
                  : launch_one<MODE_FINAL, false>(maps, kf, io, sp, plan, grid, s);
}

}  // namespace atsat
