// Device glue for resident multi-iteration runs: the boundary conditions BC_Sat applies between
// RK4 steps (planet/BoundaryConditions.h:150-518 with BC_Sat.cpp:61-179), on the fields of the dycore.
//
// Each of the three routines only moves data along one grid direction, so each is one kernel whose
// threads own disjoint lines: bcTheta works along j for every (i, k), bcPhi along k for every (i, j),
// bcRadius (with the rigid-wall u, the top taper and the species lid / wall copies) along i for
// every (j, k). They run in the order cSaturnModel::Run calls them (cSaturnModel.cpp:1091-1093).
#include "dyn_common.cuh"

namespace atsat {

namespace {

struct BCArgs {
    double* radius[20];      // bc_fields_radius() restricted to the dycore; bcPhi uses the same list
    int n_radius;
    int u_slot;              // index of u in radius[] (keeps the radial form at the bottom)
    double* theta_extrap[17];
    int n_theta_extrap;
    double* theta_zero[3];
    double* turb[3];
    double turb_floor[3];
    int turb_on;
    double* species[11];
    double* u;
    double* v;
    double* w;
    const double* rho_mix;
    double r_mix;
    int radius_form, bottom_form, pole_form, pole_fill, lid_u, top_taper, lid_copy, wall_copy, local_rho;
};

__device__ __forceinline__ double form3(int form, double a, double b, double c, double c43, double c13) {
    const int f = (form == 0) ? 3 : form;
    if (f == 1) return a;
    if (f == 2) return c43 * a - c13 * b;
    return c - 3.0 * b + 3.0 * a;
}

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

__global__ void bc_theta_kernel(const KConst K, const BCArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = 1 + blockIdx.y;
    if (k > K.km - 2 || i > K.im - 2) return;
    const int64_t kp = K.kp, jm = K.jm;
    const int64_t base = (int64_t)i * K.plane + k;     // (i, 0, k)
    auto at = [&](int j) { return base + (int64_t)j * kp; };
    if (A.pole_fill) {
        const int jf = 2;
        const double ramp = 1.0 / 2.0;
        for (int q = 0; q < A.n_theta_extrap; q++) {
            double* f = A.theta_extrap[q];
            f[at(1)] = f[at(jf)];
            f[at(jm - 2)] = f[at(jm - 1 - jf)];
        }
        for (int q = 0; q < 3; q++) {
            double* f = A.theta_zero[q];
            f[at(1)] = ramp * f[at(jf)];
            f[at(jm - 2)] = ramp * f[at(jm - 1 - jf)];
        }
        if (A.turb_on)
            for (int q = 0; q < 3; q++) {
                double* f = A.turb[q];
                f[at(1)] = smax(A.turb_floor[q], f[at(jf)]);
                f[at(jm - 2)] = smax(A.turb_floor[q], f[at(jm - 1 - jf)]);
            }
    }
    for (int q = 0; q < 3; q++) {
        A.theta_zero[q][at(0)] = 0.0;
        A.theta_zero[q][at(jm - 1)] = 0.0;
    }
    for (int q = 0; q < A.n_theta_extrap; q++) {
        double* f = A.theta_extrap[q];
        f[at(0)] = form3(A.pole_form, f[at(1)], f[at(2)], f[at(3)], K.c43, K.c13);
        f[at(jm - 1)] = form3(A.pole_form, f[at(jm - 2)], f[at(jm - 3)], f[at(jm - 4)], K.c43, K.c13);
    }
    if (A.turb_on)
        for (int q = 0; q < 3; q++) {
            double* f = A.turb[q];
            f[at(0)] = smax(A.turb_floor[q], K.c43 * f[at(1)] - K.c13 * f[at(2)]);
            f[at(jm - 1)] = smax(A.turb_floor[q], K.c43 * f[at(jm - 2)] - K.c13 * f[at(jm - 3)]);
        }
}

__global__ void bc_phi_kernel(const KConst K, const BCArgs A) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;     // i * jm + j
    if (row >= K.im * K.jm) return;
    const int64_t c0 = (int64_t)row * K.kp, c1 = c0 + K.km - 1;
    for (int q = 0; q < A.n_radius; q++) A.radius[q][c1] = A.radius[q][c0];
    if (A.turb_on)
        for (int q = 0; q < 3; q++) {
            double* f = A.turb[q];
            const double x = smax(A.turb_floor[q], f[c0]);
            f[c0] = x;
            f[c1] = x;
        }
}

__global__ void bc_radius_kernel(const KConst K, const BCArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (k >= K.km || j >= K.jm) return;
    const int64_t P = K.plane;
    const int64_t c0 = (int64_t)j * K.kp + k;                  // (0, j, k)
    const int im = K.im;
    auto at = [&](int i) { return c0 + (int64_t)i * P; };
    if (j >= 1 && j <= K.jm - 2 && k <= K.km - 2) {
        for (int q = 0; q < A.n_radius; q++) {
            double* f = A.radius[q];
            const int fb = (A.bottom_form != 0 && q != A.u_slot) ? A.bottom_form : A.radius_form;
            f[at(0)] = form3(fb, f[at(1)], f[at(2)], f[at(3)], K.c43, K.c13);
            f[at(im - 1)] = form3(A.radius_form, f[at(im - 2)], f[at(im - 3)], f[at(im - 4)], K.c43, K.c13);
        }
        if (A.turb_on)
            for (int q = 0; q < 3; q++) {
                double* f = A.turb[q];
                f[at(0)] = smax(A.turb_floor[q], K.c43 * f[at(1)] - K.c13 * f[at(2)]);
                f[at(im - 1)] = smax(A.turb_floor[q], K.c43 * f[at(im - 2)] - K.c13 * f[at(im - 3)]);
            }
    }
    if (A.lid_u) { A.u[at(0)] = 0.0; A.u[at(im - 1)] = 0.0; }
    if (A.top_taper) {
        const int iml = im - 1;
        A.v[at(iml)] = 0.0;
        A.w[at(iml)] = 0.0;
        if (A.top_taper == 2) {
            A.v[at(iml - 1)] = (1.0 / 3.0) * A.v[at(iml - 3)];
            A.w[at(iml - 1)] = (1.0 / 3.0) * A.w[at(iml - 3)];
            A.v[at(iml - 2)] = (2.0 / 3.0) * A.v[at(iml - 3)];
            A.w[at(iml - 2)] = (2.0 / 3.0) * A.w[at(iml - 3)];
        } else {
            A.v[at(iml - 1)] *= (1.0 / 3.0);
            A.w[at(iml - 1)] *= (1.0 / 3.0);
            A.v[at(iml - 2)] *= (2.0 / 3.0);
            A.w[at(iml - 2)] *= (2.0 / 3.0);
        }
    }
    if (A.lid_copy == 0 && A.wall_copy == 0) return;
    double fr = 1.0;
    if (A.wall_copy == 2) {
        double r0 = A.r_mix, r1 = A.r_mix;
        if (A.local_rho) {
            const double a = A.rho_mix[at(0)], b = A.rho_mix[at(1)];
            r0 = (a > 0.0 && isfinite(a)) ? a : A.r_mix;
            r1 = (b > 0.0 && isfinite(b)) ? b : A.r_mix;
        }
        fr = r0 / r1;
    }
    for (int q = 0; q < 11; q++) {
        double* f = A.species[q];
        if (A.lid_copy != 0) f[at(im - 1)] = f[at(im - 2)];
        if (A.wall_copy != 0) f[at(0)] = f[at(1)] * fr;
    }
}

}  // namespace

cudaError_t launch_boundary_conditions(const KConst& kc, const atsat_dyn_params& p, double* const* f,
                                       cudaStream_t s) {
    BCArgs A{};
    const int radius[20] = {ATSAT_F_T, ATSAT_F_U, ATSAT_F_V, ATSAT_F_W, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                            ATSAT_F_CH4_ICE, ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S,
                            ATSAT_F_NH3, ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_NH4SH,
                            ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH,
                            ATSAT_F_FLUXLIM_NH4SH, ATSAT_F_THERMALMASSFLUX};
    const int theta_extrap[17] = {ATSAT_F_T, ATSAT_F_U, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD, ATSAT_F_CH4_ICE,
                                  ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                                  ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_NH4SH, ATSAT_F_MASSFLUX_H2S,
                                  ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH, ATSAT_F_THERMALMASSFLUX};
    const int theta_zero[3] = {ATSAT_F_V, ATSAT_F_W, ATSAT_F_FLUXLIM_NH4SH};
    const int turb[3] = {ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_NUE};
    const int species[11] = {ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                             ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                             ATSAT_F_CH4_ICE, ATSAT_F_NH4SH};
    A.n_radius = 20;
    A.u_slot = 1;
    for (int q = 0; q < 20; q++) A.radius[q] = f[radius[q]];
    A.n_theta_extrap = 17;
    for (int q = 0; q < 17; q++) A.theta_extrap[q] = f[theta_extrap[q]];
    for (int q = 0; q < 3; q++) A.theta_zero[q] = f[theta_zero[q]];
    for (int q = 0; q < 3; q++) A.turb[q] = f[turb[q]];
    A.turb_floor[0] = 0.0;
    A.turb_floor[1] = 1.0e-10;
    A.turb_floor[2] = 0.0;
    A.turb_on = p.turb_active;
    for (int q = 0; q < 11; q++) A.species[q] = f[species[q]];
    A.u = f[ATSAT_F_U];
    A.v = f[ATSAT_F_V];
    A.w = f[ATSAT_F_W];
    A.rho_mix = f[ATSAT_F_RHO_MIX];
    A.r_mix = p.r_mix;
    A.radius_form = p.bc_radius_form;
    A.bottom_form = p.bc_bottom_form;
    A.pole_form = p.bc_pole_form;
    A.pole_fill = p.bc_pole_fill;
    A.lid_u = p.bc_lid_u;
    A.top_taper = p.bc_top_taper;
    A.lid_copy = p.bc_species_lid_copy;
    A.wall_copy = p.bc_species_wall_copy;
    A.local_rho = p.local_rho;
    bc_theta_kernel<<<dim3((kc.km - 1 + 127) / 128, kc.im - 2), 128, 0, s>>>(kc, A);
    bc_phi_kernel<<<(kc.im * kc.jm + 127) / 128, 128, 0, s>>>(kc, A);
    bc_radius_kernel<<<dim3((kc.km + 127) / 128, kc.jm), 128, 0, s>>>(kc, A);
    return cudaGetLastError();
}

}  // namespace atsat
