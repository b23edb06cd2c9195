// Radial-march RK stage of the momentum and temperature equations (rhs_u, rhs_v, rhs_w, rhs_t:
// RHS_Sat_Turb.cpp:300-560 with the stage handling of RungeKutta_Sat_Turb.cpp:250-375), the partner of
// the tracer kernel in rk_tracer_tile.cu (species_divu off). Same arithmetic as rk_mom_tile.cu, term by
// term; what differs is how the stencils reach the threads.
//
// A block owns 32 x 8 columns (k, j) and marches through a run of `plan.levels` radial levels i (the
// grid's z dimension splits i = 1 .. im-2 into runs). Its producer lane streams two kinds of group:
//   halo group of plane i: one 40 x 10 plane (theta halo of one row, phi halo of four columns so that the
//     copy starts on a 16-byte boundary) of every stencil array, plus the periodic seam column when the
//     plane does not hold it;
//   point group of level i: the level's column geometry (one contiguous copy of eight ColGeoF) and a
//     32 x 8 plane of every point input (frozen terms, sources, at the final stage dl_1 and dl_2).
// One mbarrier per group and slot. The consumers (eight warps: row j, lane k) keep every stencil array's
// values at i-1 and i in registers; per level they take the centre at i+1 from the next plane and the
// four horizontal neighbours from the current plane, so an array costs five shared loads per cell and
// each plane crosses L2 -> shared memory once (the halo boxes of rk_mom_tile.cu carry each plane twice,
// their radial neighbours included).
//
// Halo ring: 4 slots (the consumers hold planes i and i+1, the producer fills i+2 and i+3); point ring:
// 3 slots at the intermediate stages, 2 at the final stage (which also streams dl_1 and dl_2). About
// 107 KB of shared memory: two blocks (18 warps) per SM.
#include <cuda.h>

#include "mixed_physics.cuh"
#include "tma_pipe.cuh"

namespace atsat {

namespace {

using namespace mixed;
using namespace tma;

constexpr int PW = TILE_BX;                       // 40 floats per plane row
constexpr int PLANE_F = TILE_BX * TILE_BY;        // 400
constexpr int PLANE_PAD = 416;                    // the seam column starts on a 128-byte boundary
constexpr int SEAM_F = TILE_SEAM_X * TILE_J;      // 32
constexpr int HP_F = PLANE_PAD + SEAM_F;          // 448 floats = 1792 bytes per stencil array
constexpr int PT_F = TILE_K * TILE_J;             // 256 floats per point plane
constexpr int GEO_F = TILE_J * 16;                // 128 floats: eight ColGeoF
constexpr uint32_t PLANE_BYTES = PLANE_F * 4, SEAM_BYTES = SEAM_F * 4, PT_BYTES = PT_F * 4, GEO_BYTES = GEO_F * 4;
constexpr int NCW = TILE_J;
constexpr int THREADS = (NCW + 1) * 32;
constexpr int NHA_MAX = 9;
static_assert((HP_F * 4) % 128 == 0 && (PLANE_PAD * 4) % 128 == 0 && (PT_BYTES % 128) == 0 && GEO_BYTES % 128 == 0,
              "slot alignment");
static_assert(PLANE_PAD >= PLANE_F, "plane padding");

// The rings of one launch. Regular: 4 halo slots and 3 point slots (2 at the final stage), two blocks per
// SM. Compact (intermediate stages with at most 12 point arrays): 3 halo slots and 2 point slots in 74 KB,
// three blocks per SM, its producer issuing H0 H1 P0 H2 P1 ... The consumers free the slot of plane m+1 at
// the end of level m, so with either ring size and either order each group is issued a level before the
// level that reads it (tests/test_march_rings.py replays both schedules).
template <int MODE, bool CMP>
struct Shape {
    static constexpr int NHG = CMP ? 3 : 4;                                         // halo slots
    static constexpr int NPG = CMP ? 2 : ((MODE == MODE_FINAL) ? 2 : 3);            // point slots
    static constexpr int NPT = (MODE == MODE_FINAL) ? MARCH_MAX_PT : (CMP ? 12 : 14);
    static constexpr int PG_F = GEO_F + NPT * PT_F;
    static constexpr int HG_F = NHA_MAX * HP_F;
    static constexpr size_t SMEM = (size_t)(NHG * HG_F + NPG * PG_F) * 4 + 2 * (NHG + NPG) * 8;
};
static_assert(Shape<MODE_STAGE, false>::SMEM <= 113 * 1024 && Shape<MODE_FINAL, false>::SMEM <= 113 * 1024,
              "two blocks per SM");
static_assert(Shape<MODE_STAGE, true>::SMEM <= 74 * 1024, "three blocks per SM");

// point items before the optional ones
enum { P_NUE = 0, P_DPR, P_GU, P_BAN, P_BPS, P_DPTH, P_GV, P_DPPH, P_GW, P_DPS, N_PT_FIXED };

// the six raw differences of one stencil array at the centre o: radial from registers (prv, cur and the
// centre of the next plane, returned in nxt), theta and phi from the current plane
__device__ __forceinline__ void d7m(const float* hc, const float* hn, int o, int ow, int oe, float prv, float cur,
                                    float& nxt, float* e) {
    nxt = hn[o];
    const float tp = hc[o + PW], tn = hc[o - PW];
    const float pe = hc[oe], pw = hc[ow];
    e[0] = nxt - prv;
    e[1] = nxt - 2.0f * cur + prv;
    e[2] = tp - tn;
    e[3] = tp - 2.0f * cur + tn;
    e[4] = pe - pw;
    e[5] = pe - 2.0f * cur + pw;
}

__device__ __forceinline__ bool wait_warp(uint32_t bar, uint32_t parity, long long limit) {
    const bool ok = mbar_wait(bar, parity, limit);
    return !__any_sync(0xffffffffu, !ok);
}

// one tendency of u, v, w or t (never tke / dis): the next increment, or y_{n+1} with dl_1 and dl_2 from
// the level's point planes and y_n in FP64 (as mixed_physics.cuh's emit)
template <int MODE>
__device__ __forceinline__ void put(const MixedIO& io, const StageParams& sp, int q, int64_t c, float r, float dl_c,
                                    float dl1, float dl2, double yn64) {
    if (MODE == MODE_STAGE) {
        io.dl_out[q][c] = sp.c_in_f * r;
        return;
    }
    const float inc = THIRD * (dl1 + 2.0f * dl2 + dl_c) + sp.sixth_dt_f * r;
    const double y = yn64 + f2d(inc);
    io.out64[q][c] = y;
    if (io.out32[q]) {
        const float hi = d2f(y);
        io.out32[q][c] = hi;
        if (q == ATSAT_F_W && io.wlo_out) io.wlo_out[c] = d2f(y - f2d(hi));
    }
    if (sp.write_all_rhs || q < 3) io.rhs[q][c] = f2d(r);
}

template <int MODE, bool HAS_DL, bool CMP>
__global__ void __launch_bounds__(THREADS, (CMP ? 3 : 2))
rk_mom_march_kernel(const __grid_constant__ CUtensorMap map_plane, const __grid_constant__ CUtensorMap map_seam,
                    const __grid_constant__ CUtensorMap map_pt, const MixedConstF K, const MixedIO io,
                    const StageParams sp, const MarchPlan plan) {
    using S = Shape<MODE, CMP>;
    constexpr int NHG = S::NHG;
    constexpr int NPG = S::NPG;
    constexpr int DL = HAS_DL ? 1 : 0;
    constexpr int hU = 0, hV = 1 + DL, hW = 2 + 2 * DL, hT = 4 + 3 * DL, NHA = 5 + 4 * DL;
    extern __shared__ __align__(128) float smem[];
    float* hs = smem;
    float* ps = hs + NHG * S::HG_F;
    uint64_t* bars = reinterpret_cast<uint64_t*>(ps + NPG * S::PG_F);
    const Ring rh{smem_u32(bars), smem_u32(bars + NHG)};
    const Ring rp{smem_u32(bars + 2 * NHG), smem_u32(bars + 2 * NHG + NPG)};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int k0 = blockIdx.x * TILE_K;
    const int j0 = 2 + blockIdx.y * TILE_J;
    const int ib = 1 + blockIdx.z * plan.levels;
    const int ie = min(ib + plan.levels, K.im - 1);   // levels ib .. ie-1
    const int nlev = ie - ib;
    if (nlev <= 0) return;
    int seam = 0, xs = 0;
    if (k0 == 0 && K.km - 2 > k0 + TILE_K + 3) { seam = 1; xs = (K.km - 2) & ~3; }
    else if (k0 > 0 && K.km - 2 >= k0 && K.km - 2 < k0 + TILE_K) { seam = 2; xs = 0; }

    if (smem_u32(smem) & 127u) {
        if (threadIdx.x == 0) atomicOr(plan.err, ERR_ALIGN);
        return;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NHG; s++) { mbar_init(rh.full(s), 1); mbar_init(rh.empty(s), NCW); }
        for (int s = 0; s < NPG; s++) { mbar_init(rp.full(s), 1); mbar_init(rp.empty(s), NCW); }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        // ---- producer: H(0), H(1), then per level m: H(m+2), P(m) (compact: H(0), H(1), P(0), then H(m+2),
        // P(m+1)); H(g) is plane ib-1+g, P(m) level ib+m ----
        if (lane == 0) {
            const int total = 2 * nlev + 2;
            const int n_issue = total - plan.withhold;
            const uint32_t hbytes = (uint32_t)NHA * (PLANE_BYTES + (seam ? SEAM_BYTES : 0u));
            const uint32_t pbytes = GEO_BYTES + (uint32_t)plan.n_pt * PT_BYTES;
            int gh = 0, gp = 0;
            bool ok = true;
            for (int n = 0; n < n_issue; n++) {
                const bool halo = CMP ? (n < 2 || (n >= 3 && ((n - 3) & 1) == 0)) : (n < 2 || ((n - 2) & 1) == 0);
                if (halo) {
                    const int s = gh % NHG;
                    if (gh >= NHG && !mbar_wait(rh.empty(s), (uint32_t)(((gh / NHG) - 1) & 1), plan.wait_limit)) {
                        ok = false;
                        break;
                    }
                    const int i = ib - 1 + gh;
                    mbar_expect_tx(rh.full(s), hbytes);
                    for (int a = 0; a < NHA; a++) {
                        const uint32_t dst = smem_u32(hs + s * S::HG_F + a * HP_F);
                        tma_load_4d(dst, &map_plane, k0 - 4, j0 - 1, i, plan.halo[a], rh.full(s));
                        if (seam) tma_load_4d(dst + PLANE_PAD * 4, &map_seam, xs, j0, i, plan.halo[a], rh.full(s));
                    }
                    gh++;
                } else {
                    const int s = gp % NPG;
                    if (gp >= NPG && !mbar_wait(rp.empty(s), (uint32_t)(((gp / NPG) - 1) & 1), plan.wait_limit)) {
                        ok = false;
                        break;
                    }
                    const int i = ib + gp;
                    float* dst = ps + s * S::PG_F;
                    mbar_expect_tx(rp.full(s), pbytes);
                    bulk_load(smem_u32(dst), io.geof + ((int64_t)i * K.jm + j0), GEO_BYTES, rp.full(s));
                    for (int a = 0; a < plan.n_pt; a++)
                        tma_load_4d(smem_u32(dst + GEO_F + a * PT_F), &map_pt, k0, j0, i, plan.pt[a], rp.full(s));
                    gp++;
                }
            }
            if (!ok) atomicOr(plan.err, ERR_PRODUCER);
            // every copy in flight lands before the block exits
            for (int m = (gh > NHG ? gh - NHG : 0); m < gh; m++)
                if (!mbar_wait(rh.full(m % NHG), (uint32_t)((m / NHG) & 1))) break;
            for (int m = (gp > NPG ? gp - NPG : 0); m < gp; m++)
                if (!mbar_wait(rp.full(m % NPG), (uint32_t)((m / NPG) & 1))) break;
        }
        return;
    }

    // ---- consumers: row j = j0 + warp, column k = k0 + lane ----
    const int j = j0 + warp, k = k0 + lane;
    const bool valid = (k <= K.km - 2) && (j <= K.jm - 3);
    const int row = (warp + 1) * PW;
    const int o = row + lane + 4;
    int ow = o - 1, oe = o + 1;
    if (k == 0)
        ow = (seam == 1) ? PLANE_PAD + warp * TILE_SEAM_X + ((K.km - 2) - xs) : row + (K.km - 2) - (k0 - 4);
    if (k == K.km - 2) oe = (seam == 2) ? PLANE_PAD + warp * TILE_SEAM_X + (0 - xs) : row + 0 - (k0 - 4);
    const int x = warp * TILE_K + lane;
    auto fail = [&]() { if (lane == 0) atomicOr(plan.err, ERR_CONSUMER); };

    // prologue: the centres of planes ib-1 and ib
    float prv[NHA], cur[NHA];
    if (!wait_warp(rh.full(0), 0u, plan.wait_limit) || !wait_warp(rh.full(1), 0u, plan.wait_limit)) { fail(); return; }
#pragma unroll
    for (int a = 0; a < NHA; a++) {
        prv[a] = hs[a * HP_F + o];
        cur[a] = hs[S::HG_F + a * HP_F + o];
    }
    slot_reads_done();                   // prv is used at level 0, after plane ib-1's slot is refilled
    __syncwarp();
    if (lane == 0) mbar_arrive(rh.empty(0));

    // ring positions: the current plane's slot, the next plane's slot and its phase parity; the point slot
    int sc = 1, sn = 2, pn = 0, sp_ = 0, pp = 0;
    int64_t c = ((int64_t)ib * K.jm + j) * K.kp + k;
    const bool rad_src = K.rad_on != 0, precip_src = K.precip_on != 0, tmf_src = K.tmf_on != 0;

    for (int m = 0; m < nlev; m++) {
        const int i = ib + m;
        double yn64[4] = {0.0, 0.0, 0.0, 0.0};
        if (MODE == MODE_FINAL && valid) {
#pragma unroll
            for (int q = 0; q < 4; q++) yn64[q] = ldd(io.yn64[q] + c);
        }
        if (!wait_warp(rh.full(sn), (uint32_t)pn, plan.wait_limit) ||
            !wait_warp(rp.full(sp_), (uint32_t)pp, plan.wait_limit)) {
            fail();
            return;
        }
        const float* Hc = hs + sc * S::HG_F;
        const float* Hn = hs + sn * S::HG_F;
        const float* Pg = ps + sp_ * S::PG_F;
        const ColGeoF& g = reinterpret_cast<const ColGeoF*>(Pg)[warp];
        auto P = [&](int n) -> float { return Pg[GEO_F + n * PT_F + x]; };
        float nxt[NHA];

        const float nue_c = P(P_NUE);
        const float nue_t = (K.turb_coupling != 0.0f && isfinite(nue_c)) ? K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
        const float nue_t_s = nue_t * K.inv_pr_t;

        // u, v, w: derivatives, transport and viscous parts
        D6f du, dv, dw;
        {
            float a[6], b[6];
            d7m(Hc + hU * HP_F, Hn + hU * HP_F, o, ow, oe, prv[hU], cur[hU], nxt[hU], a);
            if (HAS_DL) {
                d7m(Hc + (hU + 1) * HP_F, Hn + (hU + 1) * HP_F, o, ow, oe, prv[hU + 1], cur[hU + 1], nxt[hU + 1], b);
#pragma unroll
                for (int r = 0; r < 6; r++) a[r] += b[r];
            }
            scale6(a, K, du);
            d7m(Hc + hV * HP_F, Hn + hV * HP_F, o, ow, oe, prv[hV], cur[hV], nxt[hV], a);
            if (HAS_DL) {
                d7m(Hc + (hV + 1) * HP_F, Hn + (hV + 1) * HP_F, o, ow, oe, prv[hV + 1], cur[hV + 1], nxt[hV + 1], b);
#pragma unroll
                for (int r = 0; r < 6; r++) a[r] += b[r];
            }
            scale6(a, K, dv);
            d7m(Hc + hW * HP_F, Hn + hW * HP_F, o, ow, oe, prv[hW], cur[hW], nxt[hW], a);
            d7m(Hc + (hW + 1) * HP_F, Hn + (hW + 1) * HP_F, o, ow, oe, prv[hW + 1], cur[hW + 1], nxt[hW + 1], b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
            if (HAS_DL) {
                d7m(Hc + (hW + 2) * HP_F, Hn + (hW + 2) * HP_F, o, ow, oe, prv[hW + 2], cur[hW + 2], nxt[hW + 2], b);
#pragma unroll
                for (int r = 0; r < 6; r++) a[r] += b[r];
            }
            scale6(a, K, dw);
        }
        const float un = cur[hU], du_s = HAS_DL ? cur[hU + 1] : 0.0f;
        const float vn = cur[hV], dv_s = HAS_DL ? cur[hV + 1] : 0.0f;
        const float wyn = cur[hW], wn = wyn + cur[hW + 1], dw_s = HAS_DL ? cur[hW + 2] : 0.0f;
        const float tn = cur[hT], dt_s = HAS_DL ? cur[hT + 1] : 0.0f;
        const float u = un + du_s, v = vn + dv_s, w = wn + dw_s, t = tn + dt_s;
        const float adv_u = u * du.dr + v * du.dthe * g.inv_rm + w * du.dphi * g.inv_rmsinthe;
        const float adv_v = u * dv.dr + v * dv.dthe * g.inv_rm + w * dv.dphi * g.inv_rmsinthe;
        const float adv_w = u * dw.dr + v * dw.dthe * g.inv_rm + w * dw.dphi * g.inv_rmsinthe;
        const float dif_u = du.d2r + 2.0f * u * g.inv_rm2 + du.d2the * g.inv_rm2 + 4.0f * du.dr * g.inv_rm
                          + du.dthe * g.costhe_inv_rm2sinthe + du.d2phi * g.inv_rm2sinthe2;
        const float dif_v = dv.d2r + dv.dr * g.two_inv_rm + dv.d2the * g.inv_rm2
                          + dv.dthe * g.costhe_inv_rm2sinthe - g.v_metric * v
                          + dv.d2phi * g.inv_rm2sinthe2 + 2.0f * du.dthe * g.inv_rm2
                          - dw.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
        const float dif_w = dw.d2r + dw.dr * g.two_inv_rm + dw.d2the * g.inv_rm2
                          + dw.dthe * g.costhe_inv_rm2sinthe - g.v_metric * w
                          + dw.d2phi * g.inv_rm2sinthe2 + 2.0f * du.dphi * g.inv_rm2sinthe
                          + dv.dphi * 2.0f * g.costhe * g.inv_rm2sinthe2;
        // t
        D6f dtd;
        {
            float a[6], b[6];
            d7m(Hc + hT * HP_F, Hn + hT * HP_F, o, ow, oe, prv[hT], cur[hT], nxt[hT], a);
            if (HAS_DL) {
                d7m(Hc + (hT + 1) * HP_F, Hn + (hT + 1) * HP_F, o, ow, oe, prv[hT + 1], cur[hT + 1], nxt[hT + 1], b);
#pragma unroll
                for (int r = 0; r < 6; r++) a[r] += b[r];
            }
            scale6(a, K, dtd);
        }

        if (valid) {
            const float visc = K.inv_re + nue_t;
            const int pdl = plan.p_dl;
            // rhs_u
            const float dpr = P(P_DPR);
            float buoy = 0.0f;
            if (t > 0.0f && !K.hydro_buoy) {
                const float bps = P(P_BPS);
                if (tn > 0.0f) buoy = K.kb * (P(P_BAN) - bps * dt_s / (tn * t));
                else buoy = K.kb * (bps / t - K.bref_scale * d2f(ldd(io.buoy + i)));
            }
            float gu_stage = 0.0f;
            if (!K.metric_split)
                gu_stage += K.metric_on * (dv_s * (2.0f * vn + dv_s) + dw_s * (2.0f * wn + dw_s)) * g.inv_rm;
            if (K.cor_rad_on != 0.0f) gu_stage -= K.cor_rad_on * g.cor_rad_c * dw_s;
            const float rhs_u = P(P_GU) - dpr + buoy + gu_stage - adv_u + dif_u * visc;
            put<MODE>(io, sp, ATSAT_F_U, c, rhs_u, du_s, MODE == MODE_FINAL ? P(pdl) : 0.0f,
                      MODE == MODE_FINAL ? P(pdl + 1) : 0.0f, yn64[0]);
            if (MODE != MODE_STAGE) io.aux[0][c] = f2d(rhs_u + dpr);
            // rhs_v
            const float dpth = P(P_DPTH);
            const float rhs_v = P(P_GV) - dpth - adv_v - u * v * g.inv_rm
                              + dw_s * (2.0f * wn + dw_s) * g.cotanthe * g.inv_rm - g.cor_the_c * dw_s + dif_v * visc;
            put<MODE>(io, sp, ATSAT_F_V, c, rhs_v, dv_s, MODE == MODE_FINAL ? P(pdl + 2) : 0.0f,
                      MODE == MODE_FINAL ? P(pdl + 3) : 0.0f, yn64[1]);
            if (MODE != MODE_STAGE) io.aux[1][c] = f2d(rhs_v + dpth);
            // rhs_w
            const float dpph = P(P_DPPH);
            const float cor_phi = g.cor_phi_c * (g.costhe * (v - g.vbar0) + g.sinthe_true * (u - g.ubar0));
            const float rhs_w = P(P_GW) - dpph - adv_w - (w * u + v * w * g.cotanthe) * g.inv_rm + dif_w * visc - cor_phi;
            put<MODE>(io, sp, ATSAT_F_W, c, rhs_w, dw_s, MODE == MODE_FINAL ? P(pdl + 4) : 0.0f,
                      MODE == MODE_FINAL ? P(pdl + 5) : 0.0f, yn64[2]);
            if (MODE != MODE_STAGE) io.aux[2][c] = f2d(rhs_w + dpph);
            // rhs_t (RHS_Sat_Turb.cpp:460-560)
            const float pressure_t = K.coeff_energy_p * (u * (dpr + P(P_DPS)) + v * dpth + w * dpph);
            float radiation_t = 0.0f;
            if (rad_src) {
                const float rho_f = P(plan.p_rho);
                const float rho = (rho_f > 0.0f && isfinite(rho_f)) ? rho_f : K.r_mix;
                if (rho > 0.0f) {
                    radiation_t = K.rad_factor * P(plan.p_qrad) / rho;
                    if (!isfinite(radiation_t)) radiation_t = 0.0f;
                    else if (radiation_t > 0.5f) radiation_t = 0.5f;
                    else if (radiation_t < -0.5f) radiation_t = -0.5f;
                }
            }
            float precip_t = 0.0f;
            if (precip_src) {
                precip_t = K.precip_factor * P(plan.p_qprecip);
                if (!isfinite(precip_t)) precip_t = 0.0f;
                else if (precip_t > 0.5f) precip_t = 0.5f;
                else if (precip_t < -0.5f) precip_t = -0.5f;
            }
            const float diffusion_t = diffusion(dtd, g);
            float r = pressure_t - transport(u, v, w, dtd, g) + diffusion_t * K.inv_re_pr + diffusion_t * nue_t_s;
            if (tmf_src) r -= K.tmf_chem * P(plan.p_tmf);
            r = r + radiation_t + precip_t;
            put<MODE>(io, sp, ATSAT_F_T, c, r, dt_s, MODE == MODE_FINAL ? P(pdl + 6) : 0.0f,
                      MODE == MODE_FINAL ? P(pdl + 7) : 0.0f, yn64[3]);
        }

        // the current plane and the level's point group are done with (their values have gone into the
        // stores above, so every lane's loads from them are complete)
        __syncwarp();
        if (lane == 0) {
            mbar_arrive(rh.empty(sc));
            mbar_arrive(rp.empty(sp_));
        }
#pragma unroll
        for (int a = 0; a < NHA; a++) {
            prv[a] = cur[a];
            cur[a] = nxt[a];
        }
        sc = sn;
        if (++sn == NHG) { sn = 0; pn ^= 1; }
        if (++sp_ == NPG) { sp_ = 0; pp ^= 1; }
        c += K.plane;
    }
}

template <int MODE, bool HAS_DL, bool CMP>
cudaError_t launch_one(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                       const MarchPlan& plan, dim3 grid, cudaStream_t s) {
    static bool attr = false;
    constexpr size_t smem = Shape<MODE, CMP>::SMEM;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(rk_mom_march_kernel<MODE, HAS_DL, CMP>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    rk_mom_march_kernel<MODE, HAS_DL, CMP><<<grid, THREADS, smem, s>>>(
        *reinterpret_cast<const CUtensorMap*>(maps.plane1), *reinterpret_cast<const CUtensorMap*>(maps.seam1),
        *reinterpret_cast<const CUtensorMap*>(maps.pt1), kf, io, sp, plan);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_rk_mom_march(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                                const MarchPlan& plan, int mode, cudaStream_t s) {
    const int nk = (kf.km - 1 + TILE_K - 1) / TILE_K;
    const int nj = (kf.jm - 4 + TILE_J - 1) / TILE_J;
    if (nk <= 0 || nj <= 0 || kf.im < 3) return cudaSuccess;
    const bool has_dl = io.dl_in[0] != nullptr;
    const int nha = has_dl ? 9 : 5;
    const int npt_max = mode == MODE_FINAL ? Shape<MODE_FINAL, false>::NPT : Shape<MODE_STAGE, false>::NPT;
    if (mode == MODE_RHS || kf.divu_on || plan.levels < 1 || plan.n_halo != nha || plan.n_pt < N_PT_FIXED ||
        plan.n_pt > npt_max || (mode == MODE_FINAL) != (plan.p_dl >= 0) || plan.withhold < 0)
        return cudaErrorInvalidValue;
    const dim3 grid(nk, nj, (kf.im - 2 + plan.levels - 1) / plan.levels);
    if (mode == MODE_STAGE && plan.compact && plan.n_pt <= Shape<MODE_STAGE, true>::NPT)
        return has_dl ? launch_one<MODE_STAGE, true, true>(maps, kf, io, sp, plan, grid, s)
                      : launch_one<MODE_STAGE, false, true>(maps, kf, io, sp, plan, grid, s);
    if (mode == MODE_STAGE)
        return has_dl ? launch_one<MODE_STAGE, true, false>(maps, kf, io, sp, plan, grid, s)
                      : launch_one<MODE_STAGE, false, false>(maps, kf, io, sp, plan, grid, s);
    return has_dl ? launch_one<MODE_FINAL, true, false>(maps, kf, io, sp, plan, grid, s)
                  : launch_one<MODE_FINAL, false, false>(maps, kf, io, sp, plan, grid, s);
}

}  // namespace atsat
