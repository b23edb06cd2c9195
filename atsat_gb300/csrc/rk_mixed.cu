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
// * The RK4 sum needs no accumulator: the stage increments dl_1 = dt/2 k1, dl_2 = dt/2 k2, dl_3 = dt k3
//   are kept in three buffers and the final stage forms y_{n+1} = y_n + (dl_1 + 2 dl_2 + dl_3) / 3
//   + dt/6 k4 -- the increment in FP32 (the k's are FP32 quantities), the sum with y_n in FP64. tke and
//   dis, whose stage inputs are clamped, keep a running FP32 k1 + 2 k2 + 2 k3.
// * float <-> double conversions use the integer-pipe versions of dyn_common.cuh.
//
// This file holds the direct stage kernel (one thread per cell, stencils from global memory) and the
// once-per-step prepare kernel; rk_tile.cu holds the TMA-tiled stage kernel. Both stage kernels run
// the per-cell physics of mixed_physics.cuh.
#include "mixed_physics.cuh"

namespace atsat {

namespace {

using namespace mixed;

// stencils read straight from global memory (through the read-only path)
struct GlobalSrc {
    const MixedIO& io;
    int64_t c, P;
    int kp, dkw, dke;

    __device__ __forceinline__ float cyn(int q) const { return ldf(io.yn32[q] + c); }
    __device__ __forceinline__ float cdl(int q) const { return io.dl_in[q] ? ldf(io.dl_in[q] + c) : 0.0f; }
    __device__ __forceinline__ float clo() const { return ldf(io.wlo + c); }
    __device__ __forceinline__ void diff7(const float* f, float* e) const {
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
    __device__ __forceinline__ void raw6(int q, float* a) const {
        diff7(io.yn32[q], a);
        if (q == ATSAT_F_W) {
            float b[6];
            diff7(io.wlo, b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
        if (io.dl_in[q]) {
            float b[6];
            diff7(io.dl_in[q], b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
    }
};

// One thread per cell; cells outside the integrated interior are left alone (their increments are
// set once per step by the prepare kernel).
template <int MODE>
__global__ void __launch_bounds__(256) rk_stage_mixed_kernel(const MixedConstF K, const MixedIO io,
                                                             const StageParams sp) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const bool interior = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    if (!interior) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const GlobalSrc S{io, c, K.plane, K.kp, kw - k, ke - k};
    const ColGeoF g = io.geof[(int64_t)i * K.jm + j];
    const CellState cs = momentum_t<MODE>(K, io, sp, S, i, c, g);
#pragma unroll
    for (int q = ATSAT_F_H2O; q <= ATSAT_F_NH4SH; q++) scalar<MODE>(q, K, io, sp, S, c, g, cs);
    if (K.turb) {
        scalar<MODE>(ATSAT_F_TKE, K, io, sp, S, c, g, cs);
        scalar<MODE>(ATSAT_F_DIS, K, io, sp, S, c, g, cs);
    } else if (MODE == MODE_RHS || (MODE == MODE_FINAL && sp.write_all_rhs)) {
        io.rhs[ATSAT_F_TKE][c] = 0.0;
        io.rhs[ATSAT_F_DIS][c] = 0.0;
    }
}

// Split form of the same stage (species_divu off): the momentum / temperature equations in one kernel
// and the tracers in another, NG threads per cell each taking a share of the 13 tracer fields. The
// tracer threads rebuild the stage velocities from the centre values, so the two kernels share no
// intermediate data. Smaller per-thread programs (fewer registers, more resident warps) hide memory
// latency better than the fused kernel on some grids; the autotuner decides.
template <int MODE>
__global__ void __launch_bounds__(256) rk_mom_kernel(const MixedConstF K, const MixedIO io, const StageParams sp) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const bool interior = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    if (!interior) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const GlobalSrc S{io, c, K.plane, K.kp, kw - k, ke - k};
    const ColGeoF g = io.geof[(int64_t)i * K.jm + j];
    momentum_t<MODE>(K, io, sp, S, i, c, g);
}

template <int MODE, int NG>
__global__ void __launch_bounds__(256) rk_tracer_kernel(const MixedConstF K, const MixedIO io, const StageParams sp) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z / NG, grp = blockIdx.z % NG;
    if (k >= K.km || j >= K.jm) return;
    const bool interior = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    if (!interior) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const GlobalSrc S{io, c, K.plane, K.kp, kw - k, ke - k};
    const ColGeoF g = io.geof[(int64_t)i * K.jm + j];
    const CellState cs = tracer_state(K, io, S, c);
    constexpr int NT = ATSAT_F_DIS - ATSAT_F_H2O + 1;   // 13 tracer fields
    const int q0 = ATSAT_F_H2O + grp * NT / NG, q1 = ATSAT_F_H2O + (grp + 1) * NT / NG;
#pragma unroll
    for (int q = ATSAT_F_H2O; q <= ATSAT_F_DIS; q++) {
        if (q < q0 || q >= q1) continue;
        if (is_turb(q) && !K.turb) {
            if (MODE == MODE_FINAL && sp.write_all_rhs) io.rhs[q][c] = 0.0;
            continue;
        }
        scalar<MODE>(q, K, io, sp, S, c, g, cs);
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
    // dl0[0] is the stage-0 input (every cell); dl0[1], dl0[2] need live - y_n only where no stage writes
    const bool rk_cell = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    if (pr.write_yn32 || pr.any_dl0) {
        // four fields at a time, their loads issued before their stores (the FP32 stores could alias the FP64
        // loads as far as the compiler knows, so loads left between them would wait one field at a time)
        for (int q0 = 0; q0 < NPROG; q0 += 4) {
            double ynv[4], lvv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int q = q0 + u;
                const bool have = q < NPROG, dl = have && pr.dl0[0][q];
                ynv[u] = (have && ((pr.write_yn32 && pr.yn32[q]) || dl)) ? __ldg(pr.yn64[q] + c) : 0.0;
                lvv[u] = dl ? __ldg(pr.live64[q] + c) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int q = q0 + u;
                if (q >= NPROG) break;
                const bool y32 = pr.write_yn32 && pr.yn32[q];
                if (!y32 && !pr.dl0[0][q]) continue;
                const double yn = ynv[u];
                if (y32) {
                    const float hi = d2f(yn);
                    pr.yn32[q][c] = hi;
                    if (pr.yn32_b[q]) pr.yn32_b[q][c] = hi;
                    if (q == ATSAT_F_W && pr.wlo) {
                        const float lo = d2f(yn - f2d(hi));
                        pr.wlo[c] = lo;
                        if (pr.wlo_b) pr.wlo_b[c] = lo;
                    }
                }
                if (pr.dl0[0][q]) {
                    const float d0 = d2f(lvv[u] - yn);
#pragma unroll
                    for (int b = 0; b < 3; b++)
                        if (pr.dl0[b][q] && (b == 0 || !rk_cell)) pr.dl0[b][q][c] = d0;
                }
            }
        }
    }
    // the dirty point inputs, four loads in flight per thread
    for (int q0 = 0; q0 < pr.nconv; q0 += 4) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (q0 + u < pr.nconv) v[u] = __ldg(pr.conv_src[q0 + u] + c);
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (q0 + u < pr.nconv) pr.conv_dst[q0 + u][c] = d2f(v[u]);
    }
    if (pr.skip_frozen) return;

    if (!rk_cell) return;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const int64_t cw = c - k + kw, ce = c - k + ke;
    const PrepGeo* g = pr.pgeo + ((int64_t)i * K.jm + j);
    // FP64 only where terms cancel: the differences of p_dyn, p_metric and p_stat, and the balanced
    // sums gu, gv and the buoyancy anomaly. Products that only scale a difference are FP32 (the
    // stored result is FP32). Constant products per column come from the host (PrepGeo).
    const double* p = pr.p_dyn;
    const float dpdr = d2f(__ldg(p + c + P) - __ldg(p + c - P)) * pr.inv_2dr_f;
    const float dpdthe = d2f(__ldg(p + c + kp) - __ldg(p + c - kp)) * __ldg(&g->s_the_f);
    const float dpdphi = d2f(__ldg(p + ce) - __ldg(p + cw)) * __ldg(&g->s_phi_f);
    // GB300 issues two FP64 operations per SM per cycle: the FP64 work here is the five differences, the
    // meridional balance (three fmas) and the buoyancy anomaly (three), twelve operations per cell
    double dpm_the = 0.0;          // the p_metric difference along theta
    float dpmdphi = 0.0f;
    if (K.metric_split) {
        dpm_the = __ldg(pr.p_metric + c + kp) - __ldg(pr.p_metric + c - kp);
        dpmdphi = d2f(__ldg(pr.p_metric + ce) - __ldg(pr.p_metric + cw)) * __ldg(&g->s_phi_f);
    }
    // the adiabatic term only enters rhs_t's small compression work
    float dps = 0.0f;
    if (K.adiabatic) {
        dps = d2f(__ldg(pr.p_stat + c + P) - __ldg(pr.p_stat + c - P)) * pr.dps_scale_f;
        const float rho_l = d2f(__ldg(pr.rho_mix + c));
        if (K.adiabatic_rho && rho_l > 0.0f && isfinite(rho_l)) dps *= pr.r_mix_f / rho_l;
    }
    const double t = __ldg(pr.yn64[ATSAT_F_T] + c);
    const double ps = __ldg(pr.p_stat + c);
    // buoyancy: numerator B p (so that b = B p / t; stored in FP32, so formed in FP32) and the anomaly
    // B p / t - mean at t_n. p / t: the FP32 quotient q0 = p * rcp(t) corrected once in FP64,
    // q = q0 + (p - t q0) rcp(t) (relative error ~2^-44), where t and p are moderate (t in [2^-60, 2^60),
    // |p| < 2^60: no FP32 overflow); elsewhere 1/t refined by one Newton-Raphson step times B p.
    const float tf = d2f(t);
    float bps_f;
    double ban = 0.0;
    if (K.buoy_legacy) {
        const double bps = (ps + __ldg(p + c)) * pr.bnum;
        bps_f = d2f(bps);
        if (tf > 0.0f) {
            double r = f2d(__frcp_rn(tf));
            r = fma(r, fma(-t, r, 1.0), r);
            ban = bps * r;
        }
    } else {
        const float psf = d2f(ps);
        bps_f = psf * pr.bnum_f;
        if (tf > 0.0f) {
            uint32_t lo, th, ph;
            split_f64(t, lo, th);
            split_f64(ps, lo, ph);
            const uint32_t te = (th >> 20) & 0x7FFu, pe = (ph >> 20) & 0x7FFu;
            const float rf = __frcp_rn(tf);
            const double r0 = f2d(rf);
            const double buoy_i = __ldg(pr.buoy + i);
            if (te - 963u < 120u && pe < 1083u) {
                const double q0 = f2d(psf * rf);
                ban = fma(pr.bnum, fma(fma(-t, q0, ps), r0, q0), -buoy_i);
            } else {
                const double r = fma(r0, fma(-t, r0, 1.0), r0);
                ban = ps * pr.bnum * r - buoy_i;
            }
        }
    }
    // frozen parts of rhs_u, rhs_v, rhs_w at y_n (RHS_Sat_Turb.cpp:310-350, 388-399, 780-835)
    const double wn = __ldg(pr.yn64[ATSAT_F_W] + c);
    double gu = __ldg(&g->cent_rad_c);
    if (!K.metric_split) {
        const double vn = __ldg(pr.yn64[ATSAT_F_V] + c);
        // + metric (v^2 + w^2) / rm: rhs_u subtracts transport_u, which carries - metric (RHS_Sat_Turb.cpp:391-395)
        gu += (vn * vn + wn * wn) * __ldg(&g->metric_inv_rm);
    }
    if (pr.cor_rad) gu -= __ldg(&g->cor_rad_c) * wn;
    // w (w cot / r) - Coriolis cor_the w, the centrifugal and the p_metric gradient
    const double rest = K.metric_split ? fma(-dpm_the, __ldg(&g->s_the), __ldg(&g->cent_the_c)) : __ldg(&g->cent_the_c);
    const double gv = fma(wn, fma(wn, __ldg(&g->cot_rm), -__ldg(&g->cor_the_c)), rest);
    pr.fz[FZ_DPR][c] = dpdr;
    pr.fz[FZ_DPTH][c] = dpdthe;
    pr.fz[FZ_DPPH][c] = dpdphi;
    pr.fz[FZ_DPS][c] = dps;
    pr.fz[FZ_GU][c] = d2f(gu);
    pr.fz[FZ_GV][c] = d2f(gv);
    pr.fz[FZ_GW][c] = -dpmdphi;
    pr.fz[FZ_BAN][c] = d2f(ban);
    pr.fz[FZ_BPS][c] = bps_f;
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

template <int MODE>
cudaError_t launch_split_mode(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int groups,
                              cudaStream_t s) {
    const dim3 block(32, 8);
    const unsigned gx = (kf.km + 31) / 32, gy = (kf.jm + 7) / 8;
    rk_mom_kernel<MODE><<<dim3(gx, gy, kf.im), block, 0, s>>>(kf, io, sp);
    if (groups == 1) rk_tracer_kernel<MODE, 1><<<dim3(gx, gy, kf.im), block, 0, s>>>(kf, io, sp);
    else if (groups == 3) rk_tracer_kernel<MODE, 3><<<dim3(gx, gy, kf.im * 3), block, 0, s>>>(kf, io, sp);
    else rk_tracer_kernel<MODE, 13><<<dim3(gx, gy, kf.im * 13), block, 0, s>>>(kf, io, sp);
    return cudaGetLastError();
}

cudaError_t launch_rk_mom(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode, cudaStream_t s) {
    if (kf.divu_on || mode == MODE_RHS) return cudaErrorInvalidValue;
    const dim3 block(32, 8), grid((kf.km + 31) / 32, (kf.jm + 7) / 8, kf.im);
    if (mode == MODE_STAGE) rk_mom_kernel<MODE_STAGE><<<grid, block, 0, s>>>(kf, io, sp);
    else rk_mom_kernel<MODE_FINAL><<<grid, block, 0, s>>>(kf, io, sp);
    return cudaGetLastError();
}

cudaError_t launch_rk_split(const MixedConstF& kf, const MixedIO& io, const StageParams& sp, int mode, int groups,
                            cudaStream_t s) {
    if (kf.divu_on || (groups != 1 && groups != 3 && groups != 13) || mode == MODE_RHS) return cudaErrorInvalidValue;
    return mode == MODE_STAGE ? launch_split_mode<MODE_STAGE>(kf, io, sp, groups, s)
                              : launch_split_mode<MODE_FINAL>(kf, io, sp, groups, s);
}

namespace {

// The final stage's FP64 half for fields q0..q1: y_{n+1} = y_n + increment, the increment formed in FP32
// by the tiled stage kernels and left in place of dl_1 (RungeKutta_Sat_Turb.cpp:324-375), the tke / dis
// clamps, the FP64 field, its FP32 copy and, for w, the copy's low word. A stream over the RK interior.
__global__ void __launch_bounds__(256) final_combine_kernel(const MixedConstF K, const MixedIO io, int q0, int q1) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = 2 + blockIdx.y * 8 + threadIdx.y, i = 1 + blockIdx.z;
    if (k > K.km - 2 || j > K.jm - 3 || i > K.im - 2) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    // every field's loads first: the stores below could alias them as far as the compiler knows, so loads
    // issued between stores would wait for each other (one field in flight per thread)
    double yn[NPROG];
    float inc[NPROG];
#pragma unroll
    for (int q = 0; q < NPROG; q++) {
        const bool in = q >= q0 && q <= q1;
        yn[q] = in ? ldd(io.yn64[q] + c) : 0.0;
        inc[q] = in ? __ldg(io.dl1[q] + c) : 0.0f;
    }
#pragma unroll
    for (int q = 0; q < NPROG; q++) {
        if (q < q0 || q > q1) continue;
        double y = yn[q] + f2d(inc[q]);
        if (q == ATSAT_F_TKE) y = smin(smax(y, 0.0), K.tke_max_d);
        else if (q == ATSAT_F_DIS) y = smax(y, K.dis_min_d);
        io.out64[q][c] = y;
        if (io.out32[q]) {
            const float hi = d2f(y);
            io.out32[q][c] = hi;
            if (q == ATSAT_F_W && io.wlo_out) io.wlo_out[c] = d2f(y - f2d(hi));
        }
    }
}

}  // namespace

cudaError_t launch_final_combine(const MixedConstF& kf, const MixedIO& io, int q0, int q1, cudaStream_t s) {
    final_combine_kernel<<<dim3((kf.km - 1 + 31) / 32, (kf.jm - 4 + 7) / 8, kf.im - 2), dim3(32, 8), 0, s>>>(kf, io, q0,
                                                                                                          q1);
    return cudaGetLastError();
}

cudaError_t launch_mixed_prepare(const KConst& kc, const MixedPrep& pr, cudaStream_t s) {
    dim3 block(32, 8), grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    mixed_prepare_kernel<<<grid, block, 0, s>>>(kc, pr);
    return cudaGetLastError();
}

}  // namespace atsat
