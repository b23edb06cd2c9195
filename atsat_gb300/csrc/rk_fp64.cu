// FP64 drop-in kernels of RungeKuttaSat (planet/RungeKutta_Sat_Turb.cpp:110-387) and RHSSat
// (planet/RHS_Sat_Turb.cpp:25-1016).
//
// One fused kernel per RK stage: every thread owns one cell of the RK interior
// (i = 1..im-2, j = 2..jm-3, k = 0..km-2 with the periodic seam), evaluates the full right-hand side
// of the 17 prognostic fields from the stage input Y_s, folds it into the FP64 accumulator and
// writes the next stage input Y_{s+1} = y_n + c_in * rhs (the reference's pass A and pass B,
// :220-320, in one pass over memory). The last stage writes y_{n+1} = y_n + dt/6 * acc directly
// (:324-375). Y_s and Y_{s+1} live in different buffers, so no cell reads a half-updated
// neighbour -- the property the reference's separated passes exist for (:178-202).
//
// The arithmetic follows the reference's expressions. Divisions by configuration constants are
// multiplications by reciprocals formed on the host, and exp_rm (identically 1: ATSAT has no radial
// stretching) is not multiplied; both change results by at most an ulp per operation.
#include "dyn_common.cuh"

namespace atsat {

namespace {

__device__ __forceinline__ double ldg(const double* p) { return __ldg(p); }

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

template <int MODE>
__device__ __forceinline__ void emit(const StageIO<double>& io, const StageParams& sp, const KConst& K, int q,
                                     int64_t c, double r) {
    if (MODE == MODE_RHS) {
        io.rhs[q][c] = r;
        return;
    }
    double y;
    if (MODE == MODE_STAGE) {
        const double a = (sp.stage == 0) ? sp.wgt * r : io.acc[q][c] + sp.wgt * r;
        io.acc[q][c] = a;
        y = ldg(io.yn[q] + c) + sp.c_in * r;
    } else {
        const double a = io.acc[q][c] + sp.wgt * r;
        y = ldg(io.yn[q] + c) + sp.sixth_dt * a;
        if (sp.write_all_rhs || q < 3) io.rhs[q][c] = r;
    }
    if (q == ATSAT_F_TKE) y = smin(smax(y, 0.0), K.tke_max);
    else if (q == ATSAT_F_DIS) y = smax(y, K.dis_min);
    io.out[q][c] = y;
}

// The stencil of one field as raw differences: a0 = f(i+1) - f(i-1), a1 = f(i+1) - 2 f + f(i-1), and b0, b1
// along theta, c0, c1 along phi. fma(-2, x, p) equals p - 2x bit for bit (the product is exact).
struct R6 { double a0, a1, b0, b1, c0, c1; };

__device__ __forceinline__ void raw6(const double* __restrict__ f, int64_t c, int64_t plane, int kp, int dkw,
                                     int dke, R6& r) {
    const double x = ldg(f + c);
    const double rp = ldg(f + c + plane), rn = ldg(f + c - plane);
    const double tp = ldg(f + c + kp), tn = ldg(f + c - kp);
    const double pe = ldg(f + c + dke), pw = ldg(f + c + dkw);
    r.a0 = rp - rn;
    r.a1 = fma(-2.0, x, rp) + rn;
    r.b0 = tp - tn;
    r.b1 = fma(-2.0, x, tp) + tn;
    r.c0 = pe - pw;
    r.c1 = fma(-2.0, x, pe) + pw;
}

// Per-cell factors shared by every field: the advecting velocity times the stencil scales, and the
// diffusion operator's coefficient per raw difference (from the column table).
struct Fold {
    double U, V, W, dr2, dr1, dt2, dt1, dp2;
    __device__ __forceinline__ double transport(const R6& r) const { return fma(U, r.a0, fma(V, r.b0, W * r.c0)); }
    __device__ __forceinline__ double diffusion(const R6& r) const {
        return fma(dr2, r.a1, fma(dr1, r.a0, fma(dt2, r.b1, fma(dt1, r.b0, dp2 * r.c1))));
    }
};

// GB300 issues two FP64 operations per SM per cycle, and this kernel is bound by that pipe. The reference
// scales each of a field's six differences before combining them (RHS_Sat_Turb.cpp:300-1000); here the
// scales are folded into per-cell factors (Fold) and per-column coefficients (ColGeo), so a field costs its
// nine differencing operations, three for transport and five for diffusion. Every term is the reference's;
// the products are associated differently (a few ulps per term).
template <int MODE>
__global__ void __launch_bounds__(256) rk_stage_fp64_kernel(const KConst K, const StageIO<double> io,
                                                            const StageParams sp) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t plane = K.plane;
    const int kp = K.kp;
    const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
    const bool interior = (i >= 1 && i <= K.im - 2 && j >= 2 && j <= K.jm - 3 && k <= K.km - 2);
    if (!interior) {
        // Cells the step does not integrate keep their values: the stage buffer takes them once.
        if (MODE == MODE_STAGE && sp.stage == 0) {
#pragma unroll 1
            for (int q = 0; q < NPROG; q++) io.out[q][c] = ldg(io.in[q] + c);
        }
        return;
    }
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const int dkw = kw - k, dke = ke - k;

    const ColGeo* gp = io.geo + ((int64_t)i * K.jm + j);
    const double inv_rm = ldg(&gp->inv_rm), inv_rm2 = ldg(&gp->inv_rm2), inv_rmsinthe = ldg(&gp->inv_rmsinthe);
    const double cotanthe = ldg(&gp->cotanthe), costhe = ldg(&gp->costhe), v_metric = ldg(&gp->v_metric);

    const double u = ldg(io.in[ATSAT_F_U] + c);
    const double v = ldg(io.in[ATSAT_F_V] + c);
    const double w = ldg(io.in[ATSAT_F_W] + c);
    Fold fd;
    fd.U = u * K.inv_2dr;
    fd.V = v * ldg(&gp->t_the);
    fd.W = w * ldg(&gp->t_phi);
    fd.dr2 = K.inv_dr2;
    fd.dr1 = ldg(&gp->d_r1);
    fd.dt2 = ldg(&gp->d_t2);
    fd.dt1 = ldg(&gp->d_t1);
    fd.dp2 = ldg(&gp->d_p2);

    R6 ru, rv, rw;
    raw6(io.in[ATSAT_F_U], c, plane, kp, dkw, dke, ru);
    raw6(io.in[ATSAT_F_V], c, plane, kp, dkw, dke, rv);
    raw6(io.in[ATSAT_F_W], c, plane, kp, dkw, dke, rw);
    const double dpdr = (ldg(io.p_dyn + c + plane) - ldg(io.p_dyn + c - plane)) * K.inv_2dr;
    const double dpdthe = (ldg(io.p_dyn + c + kp) - ldg(io.p_dyn + c - kp)) * K.inv_2dthe;
    const double dpdphi = (ldg(io.p_dyn + c + dke) - ldg(io.p_dyn + c + dkw)) * K.inv_2dphi;

    // eddy viscosity as the momentum / scalar equations read it (RHS_Sat_Turb.cpp:577-582)
    const double nue_c = ldg(io.nue + c);
    const double nue_t = (K.turb_coupling != 0.0 && isfinite(nue_c)) ? K.turb_coupling * smax(0.0, nue_c) : 0.0;
    const double nue_t_s = nue_t * K.inv_pr_t;

    // ---- momentum (RHS_Sat_Turb.cpp:310-350, 388-399, 435-456, 700-714, 780-835) ----
    {
        const double cor_rad = ldg(&gp->cor_rad) * w;
        const double cor_the = ldg(&gp->cor_the) * w;
        const double v_cor = v - ldg(&gp->vbar0), u_cor = u - ldg(&gp->ubar0);
        const double cor_phi = ldg(&gp->cor_phi) * (costhe * v_cor + ldg(&gp->sinthe_true) * u_cor);

        double transport_u = fd.transport(ru);
        if (!K.metric_split) transport_u = transport_u - K.metric_on * (v * v + w * w) * inv_rm;
        const double transport_v = fd.transport(rv) + (u * v - w * w * cotanthe) * inv_rm;
        const double transport_w = fd.transport(rw) + (w * u + v * w * cotanthe) * inv_rm;
        // diffusion_u: 4 du/dr / rm in place of du/dr 2 / rm, and 2 u / rm^2
        const double diffusion_u = fma(fd.dr1, ru.a0, fd.diffusion(ru)) + 2.0 * u * inv_rm2;
        const double x_v2 = ldg(&gp->x_v2);
        const double diffusion_v = fd.diffusion(rv) - v_metric * v + ldg(&gp->x_v1) * ru.b0 - x_v2 * rw.c0;
        const double diffusion_w = fd.diffusion(rw) - v_metric * w + ldg(&gp->x_w1) * ru.c0 + x_v2 * rv.c0;

        double buoyancy_u = 0.0;
        const double t_c = ldg(io.in[ATSAT_F_T] + c);
        if (t_c > 0.0 && !K.hydro_buoy) {
            const double ps = ldg(io.p_stat + c);
            if (K.buoy_legacy) buoyancy_u = K.legacy_buoy * (ps + ldg(io.p_dyn + c)) / (K.rR * t_c * K.t_ref);
            else if (in_rcp_range(t_c)) buoyancy_u = K.kbuoy * ((K.buoy_c * ps) * recip_nr(t_c) - ldg(io.buoy + i));
            else buoyancy_u = K.kbuoy * (K.g * ps / (K.rR * t_c * K.t_ref) - ldg(io.buoy + i));
        }
        const double visc = K.inv_re + nue_t;
        const double rhs_u = -dpdr + buoyancy_u - transport_u + diffusion_u * visc
                           - K.cor_rad_on * K.Coriolis * cor_rad + K.centrifugal * ldg(&gp->cent_rad);
        double dpmdthe = 0.0, dpmdphi = 0.0;
        if (K.metric_split) {
            dpmdthe = (ldg(io.p_metric + c + kp) - ldg(io.p_metric + c - kp)) * K.inv_2dthe;
            dpmdphi = (ldg(io.p_metric + c + dke) - ldg(io.p_metric + c + dkw)) * K.inv_2dphi;
        }
        const double rhs_v = -(dpdthe + dpmdthe) * inv_rm - transport_v + diffusion_v * visc - K.Coriolis * cor_the
                           + K.centrifugal * ldg(&gp->cent_the);
        const double rhs_w = -(dpdphi + dpmdphi) * inv_rmsinthe - transport_w + diffusion_w * visc
                           - K.Coriolis * cor_phi;
        emit<MODE>(io, sp, K, ATSAT_F_U, c, rhs_u);
        emit<MODE>(io, sp, K, ATSAT_F_V, c, rhs_v);
        emit<MODE>(io, sp, K, ATSAT_F_W, c, rhs_w);
        if (MODE != MODE_STAGE) {
            io.aux[0][c] = rhs_u + dpdr;
            io.aux[1][c] = rhs_v + dpdthe * inv_rm;
            io.aux[2][c] = rhs_w + dpdphi * inv_rmsinthe;
        }
    }

    // flux-form factor of the species (RHS_Sat_Turb.cpp:979-1009), 0 unless ATSAT_SPECIES_DIVU
    const double sd = K.divu_on ? K.species_divu * (ru.a0 * K.inv_2dr + 2.0 * u * inv_rm + rv.b0 * ldg(&gp->t_the)
                                                    + v * cotanthe * inv_rm + rw.c0 * ldg(&gp->t_phi))
                                : 0.0;

    // ---- temperature (RHS_Sat_Turb.cpp:368-386, 409, 435-437, 611-665, 752-759) ----
    {
        double dpstatdr = 0.0;
        if (K.adiabatic) {
            dpstatdr = (ldg(io.p_stat + c + plane) - ldg(io.p_stat + c - plane)) * K.inv_2dr * K.to_nd;
            const double rho_l = ldg(io.rho_mix + c);
            if (K.adiabatic_rho && rho_l > 0.0 && isfinite(rho_l))
                dpstatdr *= in_rcp_range(rho_l) ? K.r_mix * recip_nr(rho_l) : K.r_mix / rho_l;
        }
        const double pressure_t = K.coeff_energy_p * (u * (dpdr + dpstatdr) + v * dpdthe * inv_rm
                                                      + w * dpdphi * inv_rmsinthe);
        R6 rt;
        raw6(io.in[ATSAT_F_T], c, plane, kp, dkw, dke, rt);
        const double diffusion_t = fd.diffusion(rt);
        double radiation_t = 0.0;
        if (K.rad_on) {
            const double rho_f = ldg(io.rho_mix + c);
            const double rho = (rho_f > 0.0 && isfinite(rho_f)) ? rho_f : K.r_mix;
            if (rho > 0.0) {
                radiation_t = K.rad_coupling * ldg(io.q_rad + c) * K.rad_num / (rho * K.rad_den_c);
                if (!isfinite(radiation_t)) radiation_t = 0.0;
                else if (radiation_t > 0.5) radiation_t = 0.5;
                else if (radiation_t < -0.5) radiation_t = -0.5;
            }
        }
        double precip_t = 0.0;
        if (K.precip_on) {
            precip_t = K.precip_coupling * ldg(io.q_precip + c) * K.precip_num * K.precip_den;
            if (!isfinite(precip_t)) precip_t = 0.0;
            else if (precip_t > 0.5) precip_t = 0.5;
            else if (precip_t < -0.5) precip_t = -0.5;
        }
        double rhs_t = pressure_t - fd.transport(rt) + diffusion_t * (K.inv_re_pr + nue_t_s);
        if (K.tmf_on) rhs_t = rhs_t - K.tmf_chem * ldg(io.thermalmassflux + c);
        rhs_t = rhs_t + radiation_t + precip_t;
        emit<MODE>(io, sp, K, ATSAT_F_T, c, rhs_t);
    }

    // ---- species (RHS_Sat_Turb.cpp:409-431, 457-491, 839-937) ----
    const double pc = K.precip_coupling;
#define ATSAT_SPECIES(FID, INV_SC_RE, EXTRA)                                                   \
    {                                                                                          \
        R6 r6;                                                                                 \
        raw6(io.in[FID], c, plane, kp, dkw, dke, r6);                                          \
        double r = fma(fd.diffusion(r6), (INV_SC_RE) + nue_t_s, (EXTRA) - fd.transport(r6));   \
        if (K.divu_on) r -= sd * ldg(io.in[FID] + c);                                          \
        emit<MODE>(io, sp, K, FID, c, r);                                                      \
    }
    ATSAT_SPECIES(ATSAT_F_H2O, K.inv_sc_re_h2o, pc * ldg(io.s_precip[0] + c))
    ATSAT_SPECIES(ATSAT_F_H2O_CLOUD, K.inv_sc_re_h2o, pc * ldg(io.s_precip[1] + c))
    ATSAT_SPECIES(ATSAT_F_H2O_ICE, K.inv_sc_re_h2o, pc * ldg(io.s_precip[2] + c))
    ATSAT_SPECIES(ATSAT_F_H2S, K.inv_sc_re_h2s, K.chem * ldg(io.massflux_h2s + c))
    ATSAT_SPECIES(ATSAT_F_NH3, K.inv_sc_re_nh3, K.chem * ldg(io.massflux_nh3 + c) + pc * ldg(io.s_precip[3] + c))
    ATSAT_SPECIES(ATSAT_F_NH3_CLOUD, K.inv_sc_re_nh3, pc * ldg(io.s_precip[4] + c))
    ATSAT_SPECIES(ATSAT_F_NH3_ICE, K.inv_sc_re_nh3, pc * ldg(io.s_precip[5] + c))
    ATSAT_SPECIES(ATSAT_F_CH4, K.inv_sc_re_ch4, pc * ldg(io.s_precip[6] + c))
    ATSAT_SPECIES(ATSAT_F_CH4_CLOUD, K.inv_sc_re_ch4, pc * ldg(io.s_precip[7] + c))
    ATSAT_SPECIES(ATSAT_F_CH4_ICE, K.inv_sc_re_ch4, pc * ldg(io.s_precip[8] + c))
    // nh4sh carries the flux-limiter correction (RHS_Sat_Turb.cpp:932-937)
    ATSAT_SPECIES(ATSAT_F_NH4SH, K.inv_sc_re_nh4sh, ldg(io.fluxlim_nh4sh + c) + K.chem * ldg(io.massflux_nh4sh + c))
#undef ATSAT_SPECIES

    // ---- k-omega transport (RHS_Sat_Turb.cpp:511-538) ----
    if (K.turb) {
        {
            R6 r6;
            raw6(io.in[ATSAT_F_TKE], c, plane, kp, dkw, dke, r6);
            const double r = fma(fd.diffusion(r6), K.inv_re + nue_c * K.inv_sig_k,
                                 ldg(io.tke_source + c) - fd.transport(r6));
            emit<MODE>(io, sp, K, ATSAT_F_TKE, c, r);
        }
        {
            R6 r6;
            raw6(io.in[ATSAT_F_DIS], c, plane, kp, dkw, dke, r6);
            const double r = fma(fd.diffusion(r6), K.inv_re + nue_c * K.inv_sig_w,
                                 ldg(io.dis_source + c) - fd.transport(r6));
            emit<MODE>(io, sp, K, ATSAT_F_DIS, c, r);
        }
    } else if (MODE == MODE_RHS || (MODE == MODE_FINAL && sp.write_all_rhs)) {
        io.rhs[ATSAT_F_TKE][c] = 0.0;
        io.rhs[ATSAT_F_DIS][c] = 0.0;
    }
}

// ---- computeBuoyancyRefLevel (RungeKutta_Sat_Turb.cpp:31-50): two-level deterministic reduction ----
// One block per (level, chunk of rows); a warp takes whole rows, its lanes the meridians, four at a time
// so that eight loads are in flight per lane.
constexpr int LM_CHUNKS = 16;
constexpr int LM_THREADS = 128;

// the buoyancy g p / (r_mix R_mix T t_ref) = bc p / t of one cell (bc formed on the host); false where
// the reference skips the cell (!(t > 0), non-finite b). The level mean's rows take the fast path below
// and come here only for cells outside it.
__device__ __forceinline__ bool cell_buoyancy(const KConst& K, double tc, double pc, double& b) {
    if (in_rcp_range(tc)) {
        b = (K.buoy_c * pc) * recip_nr(tc);
    } else {
        if (!(tc > 0.0)) return false;
        b = K.g * pc / (K.rR * tc * K.t_ref);
    }
    return isfinite(b);
}

// |x| < 2^512 (zero and subnormals included), finite: an exponent test on the integer pipe
__device__ __forceinline__ bool moderate(double x) {
    uint32_t lo, hi;
    split_f64(x, lo, hi);
    return ((hi >> 20) & 0x7FFu) < 1023u + 512u;
}

// GB300 issues two FP64 operations per SM per cycle, so the per-cell work is three of them: each lane
// sums p / t over its cells of a row (the Newton-Raphson reciprocal and one fma) and the row's weight
// and the constant bc are applied once per row: sum += sin(theta_j) (bc * sum_k p/t + rest), with the
// weight sum sin(theta_j) * (cells counted). Cells with t outside the reciprocal's range or a huge p
// ("rest") take the reference's own expression and skip rule. With |p| < 2^512, 1/t < 2^127 and
// |bc| < 2^256 every fast-path term and sum is finite, as the reference's isfinite test needs.
__global__ void __launch_bounds__(LM_THREADS) level_mean_partial_kernel(const KConst K, const double* __restrict__ t,
                                                                         const double* __restrict__ ps,
                                                                         const double* __restrict__ sin_j,
                                                                         double* __restrict__ partial) {
    const int i = blockIdx.x, chunk = blockIdx.y;
    const int j0 = (int)((int64_t)K.jm * chunk / LM_CHUNKS), j1 = (int)((int64_t)K.jm * (chunk + 1) / LM_CHUNKS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool bc_ok = fabs(K.buoy_c) < 0x1p256;
    double sum = 0.0, wsum = 0.0;
    for (int j = j0 + warp; j < j1; j += LM_THREADS / 32) {
        const int64_t row = ((int64_t)i * K.jm + j) * K.kp;
        double rs = 0.0, rest = 0.0;
        int cnt = 0;
        for (int k0 = 0; k0 < K.km; k0 += 128) {
            double tv[4], pv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int k = k0 + q * 32 + lane;
                tv[q] = (k < K.km) ? __ldg(t + row + k) : 0.0;
                pv[q] = (k < K.km) ? __ldg(ps + row + k) : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (k0 + q * 32 + lane >= K.km) continue;
                if (bc_ok && in_rcp_range(tv[q]) && moderate(pv[q])) {
                    rs = fma(pv[q], recip_nr(tv[q]), rs);
                    cnt++;
                } else {
                    double b;
                    if (cell_buoyancy(K, tv[q], pv[q], b)) {
                        rest += b;
                        cnt++;
                    }
                }
            }
        }
        const double wgt = __ldg(sin_j + j);
        sum = fma(wgt, fma(K.buoy_c, rs, rest), sum);
        wsum = fma(wgt, (double)cnt, wsum);
    }
    __shared__ double s_sum[LM_THREADS / 32], s_w[LM_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        wsum += __shfl_down_sync(0xffffffffu, wsum, o);
    }
    if (lane == 0) { s_sum[warp] = sum; s_w[warp] = wsum; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < LM_THREADS / 32; q++) { a += s_sum[q]; b += s_w[q]; }
        partial[((int64_t)i * LM_CHUNKS + chunk) * 2 + 0] = a;
        partial[((int64_t)i * LM_CHUNKS + chunk) * 2 + 1] = b;
    }
}

__global__ void level_mean_final_kernel(const KConst K, const double* __restrict__ partial, double* __restrict__ buoy) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K.im) return;
    double s = 0.0, w = 0.0;
    for (int q = 0; q < LM_CHUNKS; q++) {
        s += partial[((int64_t)i * LM_CHUNKS + q) * 2 + 0];
        w += partial[((int64_t)i * LM_CHUNKS + q) * 2 + 1];
    }
    buoy[i] = (w > 0.0) ? s / w : 0.0;
}

// ---- computeMetricPressure (RungeKutta_Sat_Turb.cpp:60-108): one radial trapezoid scan per column ----
// The scan is serial in i; the loads of eight levels are issued ahead of the dependent sums. inv_rm holds
// 1 / rm(i) (a product instead of the reference's quotient: at most one rounding apart). Six FP64 operations
// per cell (seven with p_baro): f = (v^2 + w^2) / rm + cor w as two products and two fmas, and the
// trapezoid acc += dr/2 (f_{i-1} + f_i) as one add and one fma.
constexpr int MS_BATCH = 8;

__global__ void __launch_bounds__(128) metric_scan_kernel(const KConst K, const double* __restrict__ v,
                                                          const double* __restrict__ w,
                                                          const double* __restrict__ inv_rm,
                                                          const double* __restrict__ cor_j,
                                                          const double* __restrict__ p_baro,
                                                          double* __restrict__ pm, double half_dr) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 4 + threadIdx.y;
    if (k >= K.km || j >= K.jm) return;
    const double cor = __ldg(cor_j + j);
    const int64_t c0 = (int64_t)j * K.kp + k;
    double f_prev = 0.0, acc = 0.0;
    for (int i0 = 0; i0 < K.im; i0 += MS_BATCH) {
        double vv[MS_BATCH], ww[MS_BATCH], pb[MS_BATCH];
#pragma unroll
        for (int q = 0; q < MS_BATCH; q++) {
            const int64_t c = c0 + (int64_t)(i0 + q) * K.plane;
            const bool in = i0 + q < K.im;
            vv[q] = in ? __ldg(v + c) : 0.0;
            ww[q] = in ? __ldg(w + c) : 0.0;
            pb[q] = (in && p_baro) ? __ldg(p_baro + c) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < MS_BATCH; q++) {
            const int i = i0 + q;
            if (i >= K.im) break;
            const double f = fma(fma(ww[q], ww[q], vv[q] * vv[q]), __ldg(inv_rm + i), cor * ww[q]);
            if (i > 0) acc = fma(half_dr, f_prev + f, acc);
            f_prev = f;
            pm[c0 + (int64_t)i * K.plane] = p_baro ? acc + pb[q] : acc;
        }
    }
}

// ---- computeMixtureDensity (Pressure_Sat.cpp:49-62) ----
// rho = p_stat 1e5 / (R_mix t t_ref). Where t is in [2^-60, 2^60), |p_stat| < 2^60 and the constant
// c2 = 1e5 / (R_mix t_ref) is moderate (`fast`, set by the host), rho = p_stat (c2 / t) with c2 / t the
// FP32 quotient corrected once in FP64 (q = q0 + (c2 - t q0) rcp(t), relative error ~2^-44): three FP64
// operations per cell. Elsewhere the reference's expression and skip rules.
__global__ void __launch_bounds__(256) density_kernel(const KConst K, const double* __restrict__ t,
                                                      const double* __restrict__ ps, double R_mix, double c2,
                                                      float c2f, int fast, double* __restrict__ rho) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    const double tc = __ldg(t + c), pc = __ldg(ps + c);
    uint32_t lo, th, ph;
    split_f64(tc, lo, th);
    split_f64(pc, lo, ph);
    if (fast && ((th >> 20) & 0xFFFu) - 963u < 120u && ((ph >> 20) & 0x7FFu) < 1083u) {
        const float rf = __frcp_rn(d2f(tc));
        const double q0 = f2d(c2f * rf);
        rho[c] = pc * fma(fma(-tc, q0, c2), f2d(rf), q0);
        return;
    }
    const double T = tc * K.t_ref;
    if (!(T > 0.0) || !(R_mix > 0.0)) { rho[c] = 0.0; return; }
    const double den = R_mix * T;
    const double r = in_rcp_range(den) ? (pc * 1.0e5) * recip_nr(den) : (pc * 1.0e5) / den;
    rho[c] = isfinite(r) ? r : 0.0;
}

}  // namespace

cudaError_t launch_rk_stage_fp64(const KConst& kc, const StageIO<double>& io, const StageParams& sp, int mode,
                                 cudaStream_t s) {
    dim3 block(32, 8);
    dim3 grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    if (mode == MODE_RHS) rk_stage_fp64_kernel<MODE_RHS><<<grid, block, 0, s>>>(kc, io, sp);
    else if (mode == MODE_STAGE) rk_stage_fp64_kernel<MODE_STAGE><<<grid, block, 0, s>>>(kc, io, sp);
    else rk_stage_fp64_kernel<MODE_FINAL><<<grid, block, 0, s>>>(kc, io, sp);
    return cudaGetLastError();
}

cudaError_t launch_level_mean(const KConst& kc, const double* t, const double* p_stat, const double* sin_j,
                              double* partial, double* buoy, cudaStream_t s) {
    level_mean_partial_kernel<<<dim3(kc.im, LM_CHUNKS), LM_THREADS, 0, s>>>(kc, t, p_stat, sin_j, partial);
    level_mean_final_kernel<<<(kc.im + 63) / 64, 64, 0, s>>>(kc, partial, buoy);
    return cudaGetLastError();
}

cudaError_t launch_metric_scan(const KConst& kc, const double* v, const double* w, const double* inv_rm,
                               const double* cor_j, const double* p_baro, double* p_metric, cudaStream_t s) {
    dim3 block(32, 4), grid((kc.km + 31) / 32, (kc.jm + 3) / 4);
    metric_scan_kernel<<<grid, block, 0, s>>>(kc, v, w, inv_rm, cor_j, p_baro, p_metric, 0.5 * kc.dr);
    return cudaGetLastError();
}

cudaError_t launch_density(const KConst& kc, const double* t, const double* p_stat, double R_mix, double* rho,
                           cudaStream_t s) {
    dim3 block(32, 8), grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    const double c2 = (R_mix > 0.0 && kc.t_ref > 0.0) ? 1.0e5 / (R_mix * kc.t_ref) : 0.0;
    const int fast = c2 > 0x1p-60 && c2 < 0x1p60;
    density_kernel<<<grid, block, 0, s>>>(kc, t, p_stat, R_mix, c2, (float)c2, fast, rho);
    return cudaGetLastError();
}

}  // namespace atsat
