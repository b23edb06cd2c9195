// Turbulence<cSaturnModel>::run (planet/Turbulence.h:306-329) on the device, FP64: the friction velocity, the
// floors of k* and omega*, the sources of the chosen closure (k-omega SST by default, k-omega, k-epsilon) with
// the production P_k of the curvature-corrected velocity-gradient tensor and the moist buoyancy sink of k, the
// floors and caps after the source loop, the zero-gradient copy at i = 0, the eddy-viscosity cap, the seam
// copy and the two lid corners -- pass for pass in the reference's order, one kernel per pass. ATSAT has no
// solid body (cSaturnModel.h:254-255), so the land branches are constant.
//
// Per-level and per-row factors come from the host (TurbTables) with the reference's expressions: the model's
// float layer-height table (cSaturnModel.h:1062-1074), the closure's own sine (exact-zero guard, no floor),
// inv_2dthe / rm and inv_2dphi / (rm sin). The sources loop reads only the other cells' k* and omega*, which
// no thread of it writes (the floors run as separate passes), so its result does not depend on the order.
#include "dyn_common.cuh"

namespace atsat {
namespace {

constexpr double C_NUE = 0.028, DIS_MIN = 1.0e-10;

__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ double clamp3(double x, double lo, double hi) { return (x < lo) ? lo : ((x > hi) ? hi : x); }

struct TurbArgs {
    int im, jm, km, kp, periodic, model, turb_free, curv, buoy, abl_taper, local_rho, turb_active;
    int64_t plane;
    double u_0, t_ref, g, cp_mix, r_mix, R_mix, L_m, nue_air, re_turb, nue_max, k_bg_nd, vel_star_max;
    double dr, dthe, dphi, inv_2dr, abl_height, taper_dz;
    // quotients of constants, formed once on the host
    double inv_L_m, nue_air_nd, gam_ad, tL2_pr, inv_R_mix, inv_cpR;
    double ep[3], lv[3], ls[3], t_0[3];
    TurbTables tab;
    double *u, *v, *w, *t, *rho, *tke, *dis, *tken, *disn, *nue, *tks, *dss, *prod, *vel_star;
    double *gv[3], *gc[3], *gi[3];
};

__device__ __forceinline__ int64_t cidx(const TurbArgs& A, int i, int j, int k) {
    return ((int64_t)i * A.jm + j) * A.kp + k;
}

// compute_vel_star (Turbulence.h:335-378): u_tau per (j, k), at the first fluid cell i = 1
__global__ void turb_vel_star_kernel(const TurbArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (k >= A.km || j >= A.jm) return;
    double vs = 0.05;
    if (!A.turb_free) {
        const int i_surf = (1 < A.im - 1) ? 1 : A.im - 1;
        const int64_t c = cidx(A, i_surf, j, k);
        const double v_s = A.v[c], w_s = A.w[c];
        const double vw2 = v_s * v_s + w_s * w_s;
        vs = !isfinite(vw2) ? 0.05 : clamp3(sqrt(0.002) * (A.u_0 * sqrt(vw2)), 0.05, A.vel_star_max);
    }
    A.vel_star[(int64_t)j * A.kp + k] = vs;
}

__device__ __forceinline__ bool interior(const TurbArgs& A, int i, int j, int k) {
    return i >= 1 && i <= A.im - 2 && j >= 1 && j <= A.jm - 2 && k >= (A.periodic ? 0 : 1) && k <= A.km - 2;
}

// the floors before the source loop (Turbulence.h:628-630, 645-650)
__global__ void __launch_bounds__(256) turb_clamp_in_kernel(const TurbArgs A) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (!interior(A, i, j, k)) return;
    const int64_t c = cidx(A, i, j, k);
    A.tke[c] = dmax(0.0, A.tke[c]);
    A.dis[c] = dmax(DIS_MIN, A.dis[c]);
}

__device__ void sources_cell(const TurbArgs& A, int i, int j, int k) {
    const TurbTables& T = A.tab;
    const int64_t c = cidx(A, i, j, k);
    const int64_t P = A.plane, kp = A.kp;
    const int N = A.km - 1;
    const int kw = A.periodic ? (k == 0 ? N - 1 : k - 1) : k - 1;
    const int ke = A.periodic ? (k == N - 1 ? 0 : k + 1) : k + 1;
    const int64_t cw = c - k + kw, ce = c - k + ke;
    const double rm = T.rm[i], inv_rm = T.inv_rm[i];
    const double cotanthe = T.cotanthe[j];
    const double inv_rm2dthe = T.inv_rm2dthe[i];
    const double inv_rmsinthe2dphi = T.inv_rmsinthe2dphi[(int64_t)i * A.jm + j];
    const double inv_2dr = A.inv_2dr;
    const double* u = A.u; const double* v = A.v; const double* w = A.w;
    const double* tk = A.tke; const double* ds = A.dis;
    const double dudr = (u[c + P] - u[c - P]) * inv_2dr * 1.0;
    const double dvdr = (v[c + P] - v[c - P]) * inv_2dr * 1.0;
    const double dwdr = (w[c + P] - w[c - P]) * inv_2dr * 1.0;
    const double dudthe = (u[c + kp] - u[c - kp]) * inv_rm2dthe;
    const double dvdthe = (v[c + kp] - v[c - kp]) * inv_rm2dthe;
    const double dwdthe = (w[c + kp] - w[c - kp]) * inv_rm2dthe;
    const double dudphi = (u[ce] - u[cw]) * inv_rmsinthe2dphi;
    const double dvdphi = (v[ce] - v[cw]) * inv_rmsinthe2dphi;
    const double dwdphi = (w[ce] - w[cw]) * inv_rmsinthe2dphi;
    const double tkc = tk[c], dsc = ds[c];
    const double dtkedr = (tk[c + P] - tk[c - P]) * inv_2dr * 1.0;
    const double ddisdr = (ds[c + P] - ds[c - P]) * inv_2dr * 1.0;
    double cnue;
    {
        const double dis_here = dmax(dsc, DIS_MIN);
        const double tke_here = dmax(tkc, 0.0);
        cnue = (A.model == 0) ? qdiv(C_NUE * tke_here * tke_here, dis_here) : qdiv(tke_here, dis_here);
        cnue = dmin(cnue, A.nue_max);
    }
    const double u_r = A.curv ? u[c] * inv_rm : 0.0;
    const double v_r = A.curv ? v[c] * inv_rm : 0.0;
    const double w_r = A.curv ? w[c] * inv_rm : 0.0;
    const double v_cot_r = v_r * cotanthe, w_cot_r = w_r * cotanthe;
    const double g_rr = dudr, g_rt = dudthe - v_r, g_rp = dudphi - w_r;
    const double g_tr = dvdr, g_tt = dvdthe + u_r, g_tp = dvdphi - w_cot_r;
    const double g_pr = dwdr, g_pt = dwdthe, g_pp = dwdphi + u_r + v_cot_r;
    const double der = 0.66667 * (g_rr + g_tt + g_pp);
    const double prod = dmax(0.0, (cnue * (2.0 * g_rr - der) - 0.66667 * tkc) * g_rr
                                + (cnue * (g_rt + g_tr)) * g_rt
                                + (cnue * (g_rp + g_pr)) * g_rp
                                + (cnue * (2.0 * g_tt - der) - 0.66667 * tkc) * g_tt
                                + (cnue * (g_tr + g_rt)) * g_tr
                                + (cnue * (g_tp + g_pt)) * g_tp
                                + (cnue * (2.0 * g_pp - der) - 0.66667 * tkc) * g_pp
                                + (cnue * (g_pr + g_rp)) * g_pr
                                + (cnue * (g_pt + g_tp)) * g_pt);
    A.prod[c] = prod;
    const double W12 = g_rt - g_tr, W13 = g_rp - g_pr, W23 = g_tp - g_pt;
    const double Omega = sqrt(W12 * W12 + W13 * W13 + W23 * W23);
    const double L_m = A.L_m;
    double nue, tks, dss;
    if (A.model == 2) {            // compute_k_omega_SST (Turbulence.h:1020-1106)
        // GB300 issues two FP64 operations per SM per cycle and a division costs about a dozen: the
        // quotients here are products with 1 / omega, 1 / y*, 1 / CD and 1 / k (four divisions per cell
        // instead of fifteen), and those reciprocals are Newton-refined FP32 ones (qdiv) where in range
        const double a1 = 0.31, bet_star = 0.09, bet1 = 0.0333, bet2 = 0.0368, gam1 = 0.413, gam2 = 0.2, sig_w2 = 1.168;
        const double inv_bet_star = 1.0 / 0.09;
        const double nue_air_nd = A.nue_air_nd;
        const double dz_layer = dmax(1.0, T.thick_m[i - 1 > 0 ? i - 1 : 0]);
        const double y_phys = A.turb_free ? 1.0e20 : dmax(T.height_m[i] - T.height_m[0], dz_layer);
        const double y_star = y_phys * A.inv_L_m;
        const double inv_ys = qdiv(1.0, y_star), inv_ys2 = inv_ys * inv_ys;
        const double dtkedthe = (tk[c + kp] - tk[c - kp]) * inv_rm2dthe;
        const double ddisdthe = (ds[c + kp] - ds[c - kp]) * inv_rm2dthe;
        const double dtkedphi = (tk[ce] - tk[cw]) * inv_rmsinthe2dphi;
        const double ddisdphi = (ds[ce] - ds[cw]) * inv_rmsinthe2dphi;
        const double grad_dot = dtkedr * ddisdr + dtkedthe * ddisdthe + dtkedphi * ddisdphi;
        const double dis_safe = dmax(dsc, 1.0e-20);
        const double inv_dis = qdiv(1.0, dis_safe);
        const double CD_kw = dmax(2.0 * sig_w2 * inv_dis * grad_dot, 1.0e-20);
        const double sq_k = sqrt(tkc);
        const double t_a = sq_k * inv_bet_star * inv_dis * inv_ys;         // sqrt(k) / (beta* omega y*)
        const double t_b = 500.0 * nue_air_nd * inv_ys2 * inv_dis;         // 500 nu / (y*^2 omega)
        const double arg1 = dmin(dmax(t_a, t_b), qdiv(4.0 * sig_w2 * tkc * inv_ys2, CD_kw));
        const double arg2 = dmax(2.0 * t_a, t_b);
        const double a1sq = arg1 * arg1;
        const double F1 = tanh(a1sq * a1sq);
        const double F2 = tanh(arg2 * arg2);
        nue = qdiv(a1 * tkc, dmax(a1 * dis_safe, Omega * F2));
        const double tke_safe = dmax(tkc, 1.0e-20);
        const double P_k = dmin(prod, 20.0 * bet_star * tke_safe * dis_safe);
        const double Y_k = bet_star * tke_safe * dis_safe;
        const double P_w = qdiv((F1 * gam1 + (1.0 - F1) * gam2) * P_k * dis_safe, tke_safe);
        const double Y_w = (F1 * bet1 + (1.0 - F1) * bet2) * dis_safe * dis_safe;
        const double D_w = 2.0 * (1.0 - F1) * sig_w2 * inv_dis * grad_dot;
        tks = P_k - Y_k;
        dss = P_w - Y_w + D_w;
    } else if (A.model == 1) {     // compute_k_omega (Turbulence.h:929-1017)
        const double bet_star = 0.09, gam = 0.52, C_lim = 0.875, bet_0 = 0.0708;
        // the reference's quotients by rm 2 dthe, rm sin 2 dphi and 2 dr (rm + 1) as products with the
        // column's reciprocals (one division per cell)
        const double inv_r1 = qdiv(A.inv_2dr, rm + 1.0);
        const double dtkedthe = (tk[c + kp] - tk[c - kp]) * inv_rm2dthe;
        const double ddisdthe = (ds[c + kp] - ds[c - kp]) * inv_rm2dthe;
        const double dtkedphi = (tk[ce] - tk[cw]) * inv_rmsinthe2dphi;
        const double ddisdphi = (ds[ce] - ds[cw]) * inv_rmsinthe2dphi;
        const double dudr_k = (u[c + P] - u[c - P]) * inv_r1;
        const double dvdthe_k = dvdthe;
        const double dwdphi_k = dwdphi;
        const double dudthe_u = dudthe;
        const double dudphi_u = dudphi;
        const double dvdr_u = (v[c + P] - v[c - P]) * inv_r1;
        const double dwdr_u = (w[c + P] - w[c - P]) * inv_r1;
        const double dvdphi_u = dvdphi;
        const double dwdthe_u = dwdthe;
        const double S11 = dudr_k, S22 = dvdthe_k, S33 = dwdphi_k;
        const double S12 = 0.5 * (dudthe_u + dvdr_u), S13 = 0.5 * (dudphi_u + dwdr_u), S23 = 0.5 * (dvdphi_u + dwdthe_u);
        const double S_mag = sqrt(2.0 * (S11 * S11 + S22 * S22 + S33 * S33 + 2.0 * (S12 * S12 + S13 * S13 + S23 * S23)));
        const double w_hat = dmax(dsc, C_lim * S_mag / sqrt(bet_star));
        const double gd = dtkedr * ddisdr + dtkedthe * ddisdthe + dtkedphi * ddisdphi;
        const double sig_d = (gd <= 0.0) ? 0.0 : 0.125;
        const double b3 = bet_star * dmax(dsc, 1.0e-20);
        const double chi_w = fabs(qdiv(Omega * Omega * S_mag, b3 * b3 * b3));
        const double f_bet = qdiv(1.0 + 85.0 * chi_w, 1.0 + 100.0 * chi_w);
        nue = qdiv(tkc, dmax(w_hat, 1.0e-20));
        const double P_k = dmin(prod, 20.0 * bet_star * tkc * dsc);
        const double Y_k = bet_star * tkc * dsc;
        const double P_w = qdiv(gam * dsc, dmax(tkc, 1.0e-20)) * P_k;
        const double Y_w = bet_0 * f_bet * dsc * dsc;
        const double D_w = qdiv(sig_d, dmax(dsc, 1.0e-20)) * gd;
        tks = P_k - Y_k;
        dss = P_w - Y_w + D_w;
    } else {                       // compute_k_epsilon (Turbulence.h:885-926)
        const double C_eps_1 = 1.35, C_eps_2 = 1.80;
        const double y_phys = A.turb_free ? 1.0e20 : dmax(T.height_m[i] - T.height_m[0], L_m);
        const double y_star = y_phys / L_m;
        nue = C_NUE * tkc * tkc / dmax(dsc, DIS_MIN);
        const double d_plus = y_phys * A.vel_star[(int64_t)j * kp + k] / A.nue_air;
        const double f_nue = 1.0 - exp(-0.0115 * d_plus);
        const double Re_T = tkc * tkc * A.u_0 * L_m / dmax(dsc * A.nue_air, DIS_MIN * A.nue_air);
        const double f_2 = 1.0 - 0.4 / 1.8 * exp(-Re_T * Re_T / 36.0);
        nue *= f_nue;
        const double y_star2 = y_star * y_star;
        const double L_k = -2.0 * tkc / y_star2;
        const double L_w = -2.0 * dsc / y_star2 * exp(-d_plus / 2.0);
        const double tke_safe = dmax(tkc, DIS_MIN);
        const double P_w = C_eps_1 * dsc / tke_safe * prod;
        const double Y_w = C_eps_2 * f_2 * dsc * dsc / tke_safe;
        tks = prod - dsc + L_k / A.re_turb;
        dss = P_w - Y_w + L_w / A.re_turb;
    }
    // the buoyancy sink of k (Turbulence.h:800-835): B = -nu_t N^2 / Pr_t, moist N^2 in saturated cells
    if (A.buoy != 0) {
        // quotients as products with 1 / dz, 1 / T, 1 / rho and the host's constant quotients
        const double Tc = A.t[c] * A.t_ref;
        const double dz = T.height_m[i + 1] - T.height_m[i - 1];
        const double dTdz = qdiv((A.t[c + P] - A.t[c - P]) * A.t_ref, dz);
        const double inv_T = qdiv(1.0, Tc);
        double Gam = A.gam_ad, fac = 1.0;
        if (A.buoy == 3 && Tc > 0.0) {
            double rho = A.r_mix;
            if (A.local_rho) {
                const double r_ = A.rho[c];
                rho = (r_ > 0.0 && isfinite(r_)) ? r_ : A.r_mix;
            }
            double a = 0.0, b = 0.0;
            const double inv_rho = qdiv(1.0, rho);
            for (int n = 0; rho > 0.0 && n < 3; n++) {
                const double qc = (dmax(0.0, A.gc[n][c]) + dmax(0.0, A.gi[n][c])) * inv_rho;
                if (!(qc > 1.0e-9)) continue;
                const double qv = dmax(0.0, A.gv[n][c]) * inv_rho;
                const double L = Tc >= A.t_0[n] ? A.lv[n] : A.ls[n];
                a += L * qv * A.inv_R_mix * inv_T;
                b += A.ep[n] * L * L * qv * A.inv_cpR * inv_T * inv_T;
            }
            if (isfinite(a + b)) { Gam *= qdiv(1.0 + a, 1.0 + b); fac = 1.0 + a; }
        }
        const double N2 = (Tc > 0.0 && dz > 0.0) ? A.g * inv_T * (dTdz + Gam) * fac : 0.0;
        if (isfinite(N2) && (N2 > 0.0 || A.buoy == 2)) tks -= dmax(0.0, nue) * N2 * A.tL2_pr;
    }
    A.nue[c] = nue;
    A.tks[c] = tks;
    A.dss[c] = dss;
}

__global__ void __launch_bounds__(128) turb_sources_kernel(const TurbArgs A) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 4 + threadIdx.y, i = blockIdx.z;
    if (!interior(A, i, j, k)) return;
    sources_cell(A, i, j, k);
}

// the floors and caps after the source loop (Turbulence.h:634-643, 873-881)
__global__ void __launch_bounds__(256) turb_clamp_out_kernel(const TurbArgs A) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (!interior(A, i, j, k)) return;
    const int64_t c = cidx(A, i, j, k);
    const double vs = A.vel_star[(int64_t)j * A.kp + k];
    const double k_bg = A.turb_free ? A.k_bg_nd : 0.01 * vs * vs / (sqrt(C_NUE) * A.u_0 * A.u_0);
    const double tk = dmax(k_bg, A.tke[c]);
    const double ds = dmax(DIS_MIN, A.dis[c]);
    A.tke[c] = tk;
    A.dis[c] = ds;
    A.nue[c] = clamp3(A.nue[c], 0.0, A.nue_max);
    const double dsm = 20.0 * ds * ds;
    A.dss[c] = clamp3(A.dss[c], -dsm, dsm);
    const double tsm = 20.0 * tk * ds;
    A.tks[c] = clamp3(A.tks[c], -tsm, tsm);
}

// apply_wall_bc (Turbulence.h:382-423) without an obstacle: the zero-gradient copy at i = 0
__global__ void turb_wall_kernel(const TurbArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (k >= A.km || j >= A.jm) return;
    const int64_t c0 = cidx(A, 0, j, k), c1 = c0 + A.plane;
    A.tke[c0] = A.tke[c1];
    A.dis[c0] = A.dis[c1];
    A.nue[c0] = A.nue[c1];
}

// clamp_nue (Turbulence.h:564-589)
__global__ void __launch_bounds__(256) turb_nue_cap_kernel(const TurbArgs A) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y, i = blockIdx.z;
    if (k >= A.km || j >= A.jm) return;
    double f = 1.0;
    if (A.abl_taper) {
        const double z_agl = A.tab.height_m[i] - A.tab.height_m[0];
        f = clamp3((A.abl_height + A.taper_dz - z_agl) / A.taper_dz, 0.0, 1.0);
    }
    const int64_t c = cidx(A, i, j, k);
    A.nue[c] = clamp3(A.nue[c], 0.0, A.nue_max) * f;
}

// seam_copy (Turbulence.h:542-561) and fill_lid_corners (:510-540), the closure's eight arrays
__device__ __forceinline__ double* turb_array(const TurbArgs& A, int q) {
    switch (q) {
        case 0: return A.tke; case 1: return A.dis; case 2: return A.tken; case 3: return A.disn;
        case 4: return A.nue; case 5: return A.prod; case 6: return A.tks; default: return A.dss;
    }
}

__global__ void turb_seam_kernel(const TurbArgs A) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.im * A.jm * 8) return;
    const int q = e % 8, r = e / 8;
    double* a = turb_array(A, q);
    const int64_t row = (int64_t)r * A.kp;
    a[row + A.km - 1] = a[row];
}

__global__ void turb_corners_kernel(const TurbArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, q = blockIdx.y;
    if (k >= A.km) return;
    double* a = turb_array(A, q);
    const int il = A.im - 1, jm = A.jm;
    a[cidx(A, il, 0, k)] = 0.5 * (a[cidx(A, il, 1, k)] + a[cidx(A, il - 1, 0, k)]);
    a[cidx(A, il, jm - 1, k)] = 0.5 * (a[cidx(A, il, jm - 2, k)] + a[cidx(A, il - 1, jm - 1, k)]);
}

// bc_turb_active false: the lid from i = im-2 (j = 1..jm-2), then the pole rows from j = 1, jm-2 at every level
__global__ void turb_lid_kernel(const TurbArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y, q = blockIdx.z;
    if (k >= A.km || j > A.jm - 2) return;
    double* a = turb_array(A, q);
    a[cidx(A, A.im - 1, j, k)] = a[cidx(A, A.im - 2, j, k)];
}
__global__ void turb_poles_kernel(const TurbArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, q = blockIdx.z;
    if (k >= A.km || i >= A.im) return;
    double* a = turb_array(A, q);
    a[cidx(A, i, 0, k)] = a[cidx(A, i, 1, k)];
    a[cidx(A, i, A.jm - 1, k)] = a[cidx(A, i, A.jm - 2, k)];
}

}  // namespace

cudaError_t launch_turbulence(const KConst& K, const atsat_dyn_params& p, const atsat_dyn_turb_params& tp,
                              const TurbTables& tab, double* const* f, double* prod, double* vel_star, cudaStream_t s,
                              int* launches) {
    TurbArgs A{};
    A.im = K.im; A.jm = K.jm; A.km = K.km; A.kp = K.kp; A.plane = K.plane;
    A.periodic = p.phi_periodic; A.model = tp.model; A.turb_free = tp.turb_free; A.curv = tp.curv; A.buoy = tp.buoy;
    A.abl_taper = tp.abl_taper; A.local_rho = p.local_rho; A.turb_active = p.turb_active;
    A.u_0 = p.u_0; A.t_ref = p.t_ref; A.g = p.g; A.cp_mix = p.cp_mix; A.r_mix = p.r_mix; A.R_mix = p.R_mix;
    A.L_m = p.L_atm * 1.0e3;
    A.nue_air = tp.nue_gas;
    A.re_turb = tp.vel_star_ref * tp.z_0 / tp.nue_gas;
    A.nue_max = tp.nue_max_phys / (p.u_0 * A.L_m);
    A.k_bg_nd = tp.k_bg / (p.u_0 * p.u_0);
    A.vel_star_max = tp.vel_star_max;
    A.dr = tab.dr; A.dthe = tab.dthe; A.dphi = tab.dphi;
    A.inv_2dr = 1.0 / (2.0 * tab.dr);
    A.inv_L_m = 1.0 / A.L_m;
    A.nue_air_nd = A.nue_air / (A.u_0 * A.L_m);
    A.gam_ad = p.g / p.cp_mix;
    A.tL2_pr = (A.L_m / A.u_0) * (A.L_m / A.u_0) / 0.9;
    A.inv_R_mix = 1.0 / p.R_mix;
    A.inv_cpR = 1.0 / (p.cp_mix * p.R_mix);
    A.abl_height = tp.abl_height;
    A.taper_dz = tab.taper_dz;
    for (int n = 0; n < 3; n++) { A.ep[n] = tp.ep[n]; A.lv[n] = tp.lv[n]; A.ls[n] = tp.ls[n]; A.t_0[n] = tp.t_0[n]; }
    A.tab = tab;
    A.u = f[ATSAT_F_U]; A.v = f[ATSAT_F_V]; A.w = f[ATSAT_F_W]; A.t = f[ATSAT_F_T]; A.rho = f[ATSAT_F_RHO_MIX];
    A.tke = f[ATSAT_F_TKE]; A.dis = f[ATSAT_F_DIS]; A.tken = f[ATSAT_F_TKEN]; A.disn = f[ATSAT_F_DISN];
    A.nue = f[ATSAT_F_NUE]; A.tks = f[ATSAT_F_TKE_SOURCE]; A.dss = f[ATSAT_F_DIS_SOURCE];
    A.prod = prod; A.vel_star = vel_star;
    const int gv[3] = {ATSAT_F_H2O, ATSAT_F_NH3, ATSAT_F_CH4};
    const int gc[3] = {ATSAT_F_H2O_CLOUD, ATSAT_F_NH3_CLOUD, ATSAT_F_CH4_CLOUD};
    const int gi[3] = {ATSAT_F_H2O_ICE, ATSAT_F_NH3_ICE, ATSAT_F_CH4_ICE};
    for (int n = 0; n < 3; n++) { A.gv[n] = f[gv[n]]; A.gc[n] = f[gc[n]]; A.gi[n] = f[gi[n]]; }

    const dim3 b8(32, 8), g8((K.km + 31) / 32, (K.jm + 7) / 8, K.im);
    const dim3 b4(32, 4), g4((K.km + 31) / 32, (K.jm + 3) / 4, K.im);
    turb_vel_star_kernel<<<dim3((K.km + 127) / 128, K.jm), 128, 0, s>>>(A);
    turb_clamp_in_kernel<<<g8, b8, 0, s>>>(A);
    turb_sources_kernel<<<g4, b4, 0, s>>>(A);
    turb_clamp_out_kernel<<<g8, b8, 0, s>>>(A);
    turb_wall_kernel<<<dim3((K.km + 127) / 128, K.jm), 128, 0, s>>>(A);
    turb_nue_cap_kernel<<<g8, b8, 0, s>>>(A);
    *launches += 6;
    if (p.phi_periodic) {
        turb_seam_kernel<<<(K.im * K.jm * 8 + 255) / 256, 256, 0, s>>>(A);
        *launches += 1;
    }
    if (tp.turb_free) {
        if (p.turb_active) {
            turb_corners_kernel<<<dim3((K.km + 127) / 128, 8), 128, 0, s>>>(A);
            *launches += 1;
        } else {
            turb_lid_kernel<<<dim3((K.km + 127) / 128, K.jm - 2, 8), 128, 0, s>>>(A);
            turb_poles_kernel<<<dim3((K.km + 127) / 128, K.im, 8), 128, 0, s>>>(A);
            *launches += 2;
        }
    }
    return cudaGetLastError();
}

}  // namespace atsat
