// TMA-tiled RK stage of the 13 tracer fields (h2o .. nh4sh, tke, dis: RHS_Sat_Turb.cpp:580-1000 with the
// stage handling of RungeKutta_Sat_Turb.cpp:250-375), run after the momentum / temperature kernel of the
// split variant (rk_mixed.cu) when species_divu is off.
//
// A block owns 32 x 8 x 4 cells (k, j, i). A producer warp streams every array the tracers read, in the
// order the consumers use them, with tensor copies: the halo boxes (40 x 10 x 6 floats) of each field's
// y_n copy and stage increment into a 4-slot ring, and point boxes (32 x 8 x 4 floats, no halo) of the
// advecting winds, the eddy viscosity, the sources, the tke/dis running sums and, at the final stage, the
// increments dl_1 and dl_2 into a 6-slot ring. At the final stage the kernel writes the FP32 increment of
// y_{n+1} in place of dl_1 and launch_final_combine (rk_mixed.cu) adds it to y_n in FP64: the FP64 loads, adds and stores
// then stream in a kernel of their own instead of stalling the stencil kernel. Eight consumer warps (row j,
// lane k, four radial levels per lane) read everything from shared memory, so they never wait on a global
// load. A field holds at most two halo and four point slots, so a block needs 67 KB of
// shared memory and three blocks fit on an SM.
//
// The arithmetic is mixed_physics.cuh's scalar() with its constant factors folded: with the raw
// differences a0..a5 of the field (each part differenced on its own),
//   transport = (u / 2dr) a0 + (v / (2 dtheta rm)) a2 + (w / (2 dphi rm sin)) a4
//   diffusion = a1 / dr^2 + (two_inv_rm / 2dr) a0 + (inv_rm2 / dtheta^2) a3
//             + (costhe_inv_rm2sinthe / 2dtheta) a2 + (inv_rm2sinthe2 / dphi^2) a5
// (per-cell wind factors, per-column diffusion factors), r = kappa diffusion - transport + sources.
#include <cuda.h>

#include "mixed_physics.cuh"
#include "tma_pipe.cuh"

namespace atsat {

namespace {

using namespace mixed;
using namespace tma;

constexpr int TI = TTILE_I;                               // 4 radial levels per thread
constexpr int PL = TILE_BX * TILE_BY;                     // 400 floats per plane of a halo box
constexpr int BOX_F = PL * TTILE_BZ;                      // 2400
constexpr int SEAM_F = TILE_SEAM_X * TILE_J * TI;         // 128
constexpr int HSLOT_F = BOX_F + SEAM_F;                   // 2528 floats = 10112 bytes (79 x 128)
constexpr int PSLOT_F = TILE_K * TILE_J * TI;             // 1024 floats = 4096 bytes
constexpr uint32_t BOX_BYTES = BOX_F * 4, SEAM_BYTES = SEAM_F * 4, PT_BYTES = PSLOT_F * 4;
constexpr int NHS = 4, NPS = 6;                           // halo and point slots
constexpr int NCW = TILE_J;
constexpr int THREADS = (NCW + 1) * 32;
constexpr int GEO_F = TI * TILE_J * 16;                   // ColGeoF of the block's columns
constexpr int COEF_F = TI * TILE_J * 4;                   // the four per-column diffusion factors
constexpr size_t SMEM_BYTES = (size_t)NHS * HSLOT_F * 4 + (size_t)NPS * PSLOT_F * 4 + (size_t)(GEO_F + COEF_F) * 4
                            + 2 * (NHS + NPS) * 8;

static_assert((HSLOT_F * 4) % 128 == 0 && (PSLOT_F * 4) % 128 == 0 && (BOX_F * 4) % 128 == 0, "slot alignment");

// ---- the stream layout (the host builds the same, make_plan_tracer) ----
__host__ __device__ constexpr bool turb_field(int q) { return q == ATSAT_F_TKE || q == ATSAT_F_DIS; }
__host__ __device__ constexpr int n_src(int q) { return (q == ATSAT_F_NH3 || q == ATSAT_F_NH4SH) ? 2 : 1; }
template <int MODE>
__host__ __device__ constexpr int n_pt(int q) {
    return n_src(q) + (turb_field(q) ? 1 : 0) + ((MODE == MODE_FINAL && !turb_field(q)) ? 2 : 0);
}
template <bool HAS_DL>
__host__ __device__ constexpr int n_state() { return HAS_DL ? 8 : 5; }   // u, [du], v, [dv], w, wlo, [dw], nue
template <int MODE, bool HAS_DL>
__host__ __device__ constexpr int pt0(int q) {
    int n = n_state<HAS_DL>();
    for (int r = ATSAT_F_H2O; r < q; r++) n += n_pt<MODE>(r);
    return n;
}
template <bool HAS_DL>
__host__ __device__ constexpr int h0(int q) { return (q - ATSAT_F_H2O) * (HAS_DL ? 2 : 1); }

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

template <int MODE, bool HAS_DL>
__global__ void __launch_bounds__(THREADS, 3)
rk_tracer_tile_kernel(const __grid_constant__ CUtensorMap map_main, const __grid_constant__ CUtensorMap map_seam,
                      const __grid_constant__ CUtensorMap map_pt, const MixedConstF K, const MixedIO io,
                      const StageParams sp, const TracerPlan plan) {
    extern __shared__ __align__(128) float smem[];
    float* hs = smem;
    float* ps = hs + NHS * HSLOT_F;
    float* sgeo = ps + NPS * PSLOT_F;
    float* scoef = sgeo + GEO_F;
    uint64_t* bars = reinterpret_cast<uint64_t*>(scoef + COEF_F);
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
        // ---- producer: the plan's items in order, each to its ring ----
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

    // ---- consumers ----
    const int j = j0 + warp, k = k0 + lane;
    {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int e = lane + 32 * h;
            const int ii = e >> 4, f = e & 15;
            const int i = i0 + ii;
            float v = 0.0f;
            if (i < K.im && j < K.jm) v = __ldg(reinterpret_cast<const float*>(io.geof + ((int64_t)i * K.jm + j)) + f);
            sgeo[(ii * TILE_J + warp) * 16 + f] = v;
        }
        __syncwarp();
        if (lane < TI) {
            const ColGeoF& g = *reinterpret_cast<const ColGeoF*>(sgeo + (lane * TILE_J + warp) * 16);
            float* cf = scoef + (lane * TILE_J + warp) * 4;
            cf[0] = K.inv_2dr * g.two_inv_rm;
            cf[1] = K.inv_dthe2 * g.inv_rm2;
            cf[2] = K.inv_2dthe * g.costhe_inv_rm2sinthe;
            cf[3] = K.inv_dphi2 * g.inv_rm2sinthe2;
        }
        __syncwarp();
    }
    bool valid[TI];
    int c[TI], o[TI], ow[TI], oe[TI], pidx[TI];
#pragma unroll
    for (int ii = 0; ii < TI; ii++) {
        const int i = i0 + ii;
        valid[ii] = (k <= K.km - 2) && (j <= K.jm - 3) && (i <= K.im - 2);
        c[ii] = (i * K.jm + j) * K.kp + k;
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

    // ---- the winds and the eddy viscosity: point items u, [du] | v, [dv] | w, wlo, [dw] | nue ----
    float tu[TI], tv[TI], tw[TI], nts[TI], nuec[TI];
    {
        constexpr int DL = HAS_DL ? 1 : 0;
        constexpr int nU = 0, nV = 1 + DL, nW = 2 + 2 * DL, nN = 4 + 3 * DL;
        // u
        if (!wait_items<NPS>(rp, nU, nV, plan.wait_limit)) { fail(); return; }
#pragma unroll
        for (int ii = 0; ii < TI; ii++) {
            const int x = pidx[ii];
            const float u = HAS_DL ? ps[(nU % NPS) * PSLOT_F + x] + ps[((nU + 1) % NPS) * PSLOT_F + x]
                                   : ps[(nU % NPS) * PSLOT_F + x];
            tu[ii] = u * K.inv_2dr;
        }
        slot_reads_done();
        release<NPS>(rp, nU, nV);
        // v
        if (!wait_items<NPS>(rp, nV, nW, plan.wait_limit)) { fail(); return; }
#pragma unroll
        for (int ii = 0; ii < TI; ii++) {
            const int x = pidx[ii];
            const float v = HAS_DL ? ps[(nV % NPS) * PSLOT_F + x] + ps[((nV + 1) % NPS) * PSLOT_F + x]
                                   : ps[(nV % NPS) * PSLOT_F + x];
            const ColGeoF& g = *reinterpret_cast<const ColGeoF*>(sgeo + (ii * TILE_J + warp) * 16);
            tv[ii] = v * (K.inv_2dthe * g.inv_rm);
        }
        slot_reads_done();
        release<NPS>(rp, nV, nW);
        // w = (y_n + low word) + increment
        if (!wait_items<NPS>(rp, nW, nN, plan.wait_limit)) { fail(); return; }
#pragma unroll
        for (int ii = 0; ii < TI; ii++) {
            const int x = pidx[ii];
            float w = ps[(nW % NPS) * PSLOT_F + x] + ps[((nW + 1) % NPS) * PSLOT_F + x];
            if (HAS_DL) w = w + ps[((nW + 2) % NPS) * PSLOT_F + x];
            const ColGeoF& g = *reinterpret_cast<const ColGeoF*>(sgeo + (ii * TILE_J + warp) * 16);
            tw[ii] = w * (K.inv_2dphi * g.inv_rmsinthe);
        }
        slot_reads_done();
        release<NPS>(rp, nW, nN);
        // nue
        if (!wait_items<NPS>(rp, nN, nN + 1, plan.wait_limit)) { fail(); return; }
#pragma unroll
        for (int ii = 0; ii < TI; ii++) {
            const float nue_c = ps[(nN % NPS) * PSLOT_F + pidx[ii]];
            const float nue_t = (K.turb_coupling != 0.0f && isfinite(nue_c)) ? K.turb_coupling * smaxf(0.0f, nue_c) : 0.0f;
            nts[ii] = nue_t * K.inv_pr_t;
            nuec[ii] = nue_c;
        }
        slot_reads_done();
        release<NPS>(rp, nN, nN + 1);
        static_assert(nN + 1 == n_state<HAS_DL>(), "state items");
    }

    const int q_last = K.turb ? ATSAT_F_DIS : ATSAT_F_NH4SH;
    const float pc = K.precip_coupling, chem = K.chem;
#pragma unroll
    for (int q = ATSAT_F_H2O; q <= ATSAT_F_DIS; q++) {
        if (q > q_last) break;
        const int hb = h0<HAS_DL>(q), pb = pt0<MODE, HAS_DL>(q), npq = n_pt<MODE>(q);
        if (!wait_items<NHS>(rh, hb, hb + (HAS_DL ? 2 : 1), plan.wait_limit) ||
            !wait_items<NPS>(rp, pb, pb + npq, plan.wait_limit)) {
            fail();
            return;
        }
        const float* Y = hs + (hb % NHS) * HSLOT_F;
        const float* D = hs + ((hb + 1) % NHS) * HSLOT_F;
        const float* P0 = ps + (pb % NPS) * PSLOT_F;
        const float* P1 = ps + ((pb + 1) % NPS) * PSLOT_F;
        const float* P2 = ps + ((pb + 2) % NPS) * PSLOT_F;
        const float* P3 = ps + ((pb + 3) % NPS) * PSLOT_F;
        // the field's diffusivity and source weights (RHS_Sat_Turb.cpp:580-1000 via mixed_physics.cuh)
        float kap0, w0 = 0.0f, w1 = 0.0f;
        switch (q) {
            case ATSAT_F_H2O: case ATSAT_F_H2O_CLOUD: case ATSAT_F_H2O_ICE: kap0 = K.inv_sc_re_h2o; w0 = pc; break;
            case ATSAT_F_H2S: kap0 = K.inv_sc_re_h2s; w0 = chem; break;
            case ATSAT_F_NH3: kap0 = K.inv_sc_re_nh3; w0 = chem; w1 = pc; break;
            case ATSAT_F_NH3_CLOUD: case ATSAT_F_NH3_ICE: kap0 = K.inv_sc_re_nh3; w0 = pc; break;
            case ATSAT_F_CH4: case ATSAT_F_CH4_CLOUD: case ATSAT_F_CH4_ICE: kap0 = K.inv_sc_re_ch4; w0 = pc; break;
            case ATSAT_F_NH4SH: kap0 = K.inv_sc_re_nh4sh; w0 = 1.0f; w1 = chem; break;
            default: kap0 = K.inv_re; w0 = 1.0f; break;   // tke, dis: source weight 1
        }
        const float inv_sig = (q == ATSAT_F_TKE) ? K.inv_sig_k : K.inv_sig_w;
#pragma unroll
        for (int ii = 0; ii < TI; ii++) {
            if (!valid[ii]) continue;
            float a[6];
            d7(Y, o[ii], ow[ii], oe[ii], a);
            if (HAS_DL) {
                float b[6];
                d7(D, o[ii], ow[ii], oe[ii], b);
#pragma unroll
                for (int r = 0; r < 6; r++) a[r] += b[r];
            }
            const float yn_c = Y[o[ii]], dl_c = HAS_DL ? D[o[ii]] : 0.0f;
            const float* cf = scoef + (ii * TILE_J + warp) * 4;
            const float df = K.inv_dr2 * a[1] + cf[0] * a[0] + cf[1] * a[3] + cf[2] * a[2] + cf[3] * a[5];
            const float tr = tu[ii] * a[0] + tv[ii] * a[2] + tw[ii] * a[4];
            const int x = pidx[ii];
            float S = w0 * P0[x];
            if (n_src(q) == 2) S += w1 * P1[x];
            const float kap = turb_field(q) ? kap0 + nuec[ii] * inv_sig : kap0 + nts[ii];
            const float r = kap * df - tr + S;
            const int cc = c[ii];
            if (MODE == MODE_STAGE) {
                const float cr = sp.c_in_f * r;
                float d = cr;
                if (turb_field(q)) {
                    const float accv = (n_src(q) == 2 ? P2 : P1)[x];
                    io.acc_turb[q - ATSAT_F_TKE][cc] = (sp.stage == 0) ? sp.wgt_f * r : accv + sp.wgt_f * r;
                    const float y = yn_c + cr;
                    const float yc = (q == ATSAT_F_TKE) ? sminf(smaxf(y, 0.0f), K.tke_max) : smaxf(y, K.dis_min);
                    d = yc - yn_c;
                }
                io.dl_out[q][cc] = d;
            } else {
                float inc;
                if (turb_field(q)) {
                    inc = sp.sixth_dt_f * (P1[x] + r);
                } else {
                    const float dl1 = (n_src(q) == 2 ? P2 : P1)[x], dl2 = (n_src(q) == 2 ? P3 : P2)[x];
                    inc = THIRD * (dl1 + 2.0f * dl2 + dl_c) + sp.sixth_dt_f * r;
                }
                // the increment of y_{n+1}, in place of dl_1 (read above from this cell's point box);
                // launch_final_combine adds it to y_n in FP64
                io.dl1[q][cc] = inc;
                if (sp.write_all_rhs) io.rhs[q][cc] = f2d(r);
            }
        }
        release<NHS>(rh, hb, hb + (HAS_DL ? 2 : 1));
        release<NPS>(rp, pb, pb + npq);
    }
    if (!K.turb && MODE == MODE_FINAL && sp.write_all_rhs) {
#pragma unroll
        for (int ii = 0; ii < TI; ii++)
            if (valid[ii]) {
                io.rhs[ATSAT_F_TKE][c[ii]] = 0.0;
                io.rhs[ATSAT_F_DIS][c[ii]] = 0.0;
            }
    }
}

template <int MODE, bool HAS_DL>
cudaError_t launch_one(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                       const TracerPlan& plan, dim3 grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(rk_tracer_tile_kernel<MODE, HAS_DL>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    rk_tracer_tile_kernel<MODE, HAS_DL><<<grid, THREADS, SMEM_BYTES, s>>>(
        *reinterpret_cast<const CUtensorMap*>(maps.main4), *reinterpret_cast<const CUtensorMap*>(maps.seam4),
        *reinterpret_cast<const CUtensorMap*>(maps.pt4), kf, io, sp, plan);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_rk_tracer_tile(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io,
                                  const StageParams& sp, const TracerPlan& plan, int mode, cudaStream_t s) {
    const int nk = (kf.km - 1 + TILE_K - 1) / TILE_K;
    const int nj = (kf.jm - 4 + TILE_J - 1) / TILE_J;
    const int ni = (kf.im - 2 + TI - 1) / TI;
    if (nk <= 0 || nj <= 0 || ni <= 0) return cudaSuccess;
    if (mode == MODE_RHS || kf.divu_on || kf.fsz_over_int || plan.n_items > TRACER_MAX_ITEMS) return cudaErrorInvalidValue;
    const dim3 grid(nk, nj, ni);
    const bool has_dl = io.dl_in[0] != nullptr;
    if (mode == MODE_STAGE)
        return has_dl ? launch_one<MODE_STAGE, true>(maps, kf, io, sp, plan, grid, s)
                      : launch_one<MODE_STAGE, false>(maps, kf, io, sp, plan, grid, s);
    cudaError_t e = has_dl ? launch_one<MODE_FINAL, true>(maps, kf, io, sp, plan, grid, s)
                           : launch_one<MODE_FINAL, false>(maps, kf, io, sp, plan, grid, s);
    if (e != cudaSuccess) return e;
    return launch_final_combine(kf, io, ATSAT_F_H2O, kf.turb ? ATSAT_F_DIS : ATSAT_F_NH4SH, s);
}

// the number of items the kernel consumes (the host's plan must match)
int tracer_plan_items(int mode, bool has_dl, bool turb) {
    int n = has_dl ? 8 : 5;
    for (int q = ATSAT_F_H2O; q < NPROG; q++) {
        if (turb_field(q) && !turb) continue;
        n += (has_dl ? 2 : 1) + ((mode == MODE_FINAL) ? n_pt<MODE_FINAL>(q) : n_pt<MODE_STAGE>(q));
    }
    return n;
}

}  // namespace atsat
