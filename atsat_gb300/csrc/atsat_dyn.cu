// Host side of the C ABI declared in include/atsat_dyn.h.
//
// A handle owns its CUDA stream, one device allocation that holds every field in the pitched SoA
// layout of dyn_common.cuh, the per-column geometry table, and the host bindings. Compute entry
// points enqueue kernels on the handle's stream and synchronise before returning.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include <omp.h>

#include <cuda.h>

#include "dyn_common.cuh"

using namespace atsat;

namespace {

enum BindKind { BIND_NONE = 0, BIND_ARRAY = 1, BIND_ROWS = 2 };

struct ProfEvent {
    int cls;
    cudaEvent_t a, b;
};

}  // namespace

struct atsat_dyn {
    atsat_dyn_grid g{};
    std::vector<double> rad_z, the_z;
    atsat_dyn_params p{};
    KConst kc{};
    int device = 0;
    cudaStream_t stream = nullptr;

    double* slab = nullptr;              // one allocation for every device array below
    double* f[ATSAT_NFIELDS] = {};
    double* stage[NPROG] = {};
    double* acc[NPROG] = {};
    double* src = nullptr;
    // PRESS_LINE / PRESS_BAROTROPIC: forward-sweep scratch of the line pass, interior-mean partials and
    // the means on entry and after a sweep, the barotropic tables and scratch (one allocation)
    double* pv_buf = nullptr;
    // the turbulence closure: its knobs, one allocation for P_k (fsz), u_tau (jm x kp) and the tables
    atsat_dyn_turb_params tp{};
    double* turb_buf = nullptr;
    double *turb_prod = nullptr, *turb_vs = nullptr;
    TurbTables ttab{};
    // clampNegativeSpecies' budget: added[11], added_bnd[11] (doubles), cells[11], cells_bnd[11] (counts)
    double* clamp_added = nullptr;
    unsigned long long* clamp_cells = nullptr;
    double* clamp_partial = nullptr;     // the floor's per-block sums
    double *line_cp = nullptr, *line_dp = nullptr, *imean_partial = nullptr, *pmean = nullptr;
    BaroTables baro{};
    double* p_baro = nullptr;            // null unless set
    double* partial = nullptr;
    double* buoy = nullptr;
    double* sin_j = nullptr;
    double* rm_tab = nullptr;            // 1 / rm(i)
    double* cor_j = nullptr;
    ColGeo* geo = nullptr;
    double** six = nullptr;              // device array: aux_u, aux_v, aux_w, rhs_u, rhs_v, rhs_w
    unsigned long long* counter = nullptr;
    std::vector<ColGeo> geo_h;
    bool has_pbaro = false;

    int bind_kind[ATSAT_NFIELDS] = {};
    double* bind_base[ATSAT_NFIELDS] = {};
    std::vector<double*> bind_rows[ATSAT_NFIELDS];
    // ragged-row bindings: two pinned staging buffers of fsz doubles, each with the event of its last copy,
    // so that packing (unpacking) one field on the host overlaps the transfer of the one before (after)
    double* pinned[2] = {};
    cudaEvent_t ev_pin[2] = {};
    int pin_next = 0;
    int rows_pending = -1, rows_pending_buf = 0;
    // copy pipeline for contiguous host arrays: two device staging buffers of im*jm*km doubles, a copy
    // stream, and per buffer an event for "copy landed / re-pitched out" and one for "free again"
    double* dstage[2] = {};
    cudaStream_t cstream = nullptr;
    // the second stream of the step's start (the metric scan beside the level mean) and its fork / join
    cudaStream_t astream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_ajoin = nullptr;
    cudaEvent_t ev_ready[2] = {}, ev_free[2] = {}, ev_join = nullptr;
    int stage_next = 0;
    // bindings the SMs move in place (host_xfer.cu): host_ok when the device addresses host memory
    // through the CPU's page tables, host_direct when that path is selected, per field whether its
    // binding takes it, and the device copy of a ragged binding's row-pointer table
    bool host_ok = false, host_direct = false;
    bool async = false;                  // entry points return without waiting (ATSAT_DYN_ASYNC)
    bool direct[ATSAT_NFIELDS] = {};
    double** dev_rows[ATSAT_NFIELDS] = {};

    int64_t launches = 0;
    bool profiling = false;
    uint32_t prof_mask = ~0u;            // the kernel classes profiled
    std::vector<ProfEvent> pend;
    std::vector<cudaEvent_t> pool;
    int64_t prof_n[ATSAT_K_NCLASS] = {};
    double prof_ms[ATSAT_K_NCLASS] = {};

    int write_all_rhs = 0;
    cudaEvent_t timer[2] = {nullptr, nullptr};

    // mixed precision: FP32 copy of y_n, two FP32 increment buffers, FP32 copies of the point inputs
    float* slab32 = nullptr;
    float* yn32[NPROG] = {};             // FP32 copy of y_n read by this step's stencils
    float* wlo = nullptr;
    float* yo32[NPROG] = {};             // the other copy: receives y_{n+1} in a resident run
    float* wlo_o = nullptr;
    // Resident mixed runs (atsat_dyn_iterate): the live and n-level FP64 fields share one buffer
    // (restoreVar makes them equal and the mixed stages never write the live fields before the final
    // update, which reads y_n only at the cell it writes), and the FP32 copies are swapped, not rebuilt.
    bool aliased = false;
    bool shadow_valid = false;
    double* spare_n[NPROG] = {};
    // while aliased: the fields whose n-level has its own storage again (spare_n) because a call after
    // restoreVar changed the live field alone (the turbulence closure: k* and omega*)
    uint32_t split_mask = 0;
    // stage increments dl_1, dl_2, dl_3 (the stage-0 input live - y_n sits in C until stage 2)
    float* dlA[NPROG] = {};
    float* dlB[NPROG] = {};
    float* dlC[NPROG] = {};
    uint32_t edges_dirty = ~0u;          // fields whose cells no stage writes may hold non-zero A, B, C
    float* acc_turb[2] = {};             // tke, dis: k1 + 2 k2 + 2 k3
    float* fz[NFZ] = {};
    float* conv32[NCONV] = {};
    bool conv_dirty[NCONV] = {};
    int64_t n32 = 0;                     // FP32 arrays of fsz floats at the head of slab32
    ColGeoF* geof = nullptr;
    PrepGeo* pgeo = nullptr;
    MixedConstF kf{};
    // the TMA-tiled stage kernels: tensor maps over slab32; the stage variant (ATSAT_DYN_STAGE_*)
    TileMaps maps{};
    bool tile_ok = false;
    int variant = 1;
    unsigned int* dev_err = nullptr;     // device status word of the bounded waits
    int timeouts = 0;
    // the bounded waits' limit in SM clocks, and the test hook that leaves the last items of each tiled
    // block's stream unissued (atsat_dyn_set_wait_test)
    long long wait_limit = TILE_WAIT_LIMIT;
    int test_withhold = 0;
    int march_levels = 0;                // radial levels per block of the march kernel (the march depth)
    bool tuned_from_cache = false;       // the variant and the march depth came from the autotune cache
    PoissonSolver* poisson = nullptr;    // standalone pressure-equation solver, built on first use
    // a captured CUDA graph of `graph_iters` resident iterations (atsat_dyn_graph_capture)
    cudaGraphExec_t graph = nullptr;
    int32_t graph_iters = 0;
    int64_t graph_kernels = 0;
    std::string err;
};

namespace {

int fail(atsat_dyn* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    return code;
}

#define CK(h, call)                                                                                     \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(h, ATSAT_DYN_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                      \
    } while (0)

cudaEvent_t ev_get(atsat_dyn* h) {
    if (!h->pool.empty()) {
        cudaEvent_t e = h->pool.back();
        h->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Bracket the launches of one kernel class with events when profiling is on.
struct Timed {
    atsat_dyn* h;
    int cls;
    cudaEvent_t a = nullptr, b = nullptr;
    Timed(atsat_dyn* h_, int cls_) : h(h_), cls(cls_) {
        if (h->profiling && ((h->prof_mask >> cls) & 1u)) {
            a = ev_get(h);
            b = ev_get(h);
            cudaEventRecord(a, h->stream);
        }
    }
    ~Timed() {
        if (a) {
            cudaEventRecord(b, h->stream);
            h->pend.push_back({cls, a, b});
        }
    }
};

int resolve_profile(atsat_dyn* h) {
    if (h->pend.empty()) return ATSAT_DYN_OK;
    CK(h, cudaStreamSynchronize(h->stream));
    for (auto& e : h->pend) {
        float ms = 0.f;
        CK(h, cudaEventElapsedTime(&ms, e.a, e.b));
        h->prof_n[e.cls] += 1;
        h->prof_ms[e.cls] += ms;
        h->pool.push_back(e.a);
        h->pool.push_back(e.b);
    }
    h->pend.clear();
    return ATSAT_DYN_OK;
}

double metric_radius(const atsat_dyn_params& p, double r) {
    const double R_km = p.metric_radius_km;
    if (!(R_km > 0.0)) return r;
    return r + (R_km / p.L_atm - 1.0);
}

int check_supported(atsat_dyn* h, const atsat_dyn_params& p) {
    struct { int bad; const char* what; } rules[] = {
        {p.phi_periodic == 0, "ATSAT_BC_PHI_PERIODIC=0 (the non-periodic seam)"},
        {p.chrom != 0, "ATSAT_CHROM (chromophore tracer)"},
        {p.cp_h2_dyn != 0, "ATSAT_CP_H2 / ATSAT_CP_GAS in the dynamics"},
        {p.print_diag != 0, "ATSAT_TB/UB/CWB_DIAG print-only accumulators"},
        {p.coord_stretching != 0, "radial coordinate stretching"},
        {p.hydro_buoy != 0, "ATSAT_HYDRO_BUOY"},
        {p.t_limiter != 0, "ATSAT_T_LIMITER (reads tn at k-1 = -1 on the periodic seam in the reference)"},
        {p.press_wall != 0, "ATSAT_PRESS_WALL (no solid body exists in ATSAT)"},
        {p.precision != ATSAT_DYN_FP64 && p.precision != ATSAT_DYN_MIXED, "unknown precision"},
        // the split Coriolis form balances against the metric pressure, which only the metric split computes;
        // the reference switches it off with the metric split (cSaturnModel.cpp's knob resolution)
        {p.coriolis_split != 0 && p.metric_split == 0, "ATSAT_CORIOLIS_SPLIT without ATSAT_METRIC_SPLIT"},
        {p.hydro_buoy != 0 && p.metric_split == 0, "ATSAT_HYDRO_BUOY without ATSAT_METRIC_SPLIT"},
    };
    for (auto& r : rules)
        if (r.bad) return fail(h, ATSAT_DYN_E_UNSUPPORTED, "not implemented on the device: %s", r.what);
    return ATSAT_DYN_OK;
}

void build_constants(atsat_dyn* h) {
    const atsat_dyn_params& p = h->p;
    const atsat_dyn_grid& g = h->g;
    KConst& K = h->kc;
    K.im = g.im; K.jm = g.jm; K.km = g.km;
    K.kp = (g.km + 31) / 32 * 32;
    K.plane = (int64_t)g.jm * K.kp;
    K.fsz = (int64_t)g.im * K.plane;
    K.periodic = p.phi_periodic;
    K.turb = p.turb_active;
    K.metric_split = p.metric_split;
    K.coriolis_split = p.coriolis_split;
    K.adiabatic = p.adiabatic;
    K.adiabatic_rho = p.adiabatic_rho;
    K.buoy_legacy = p.buoy_legacy;
    K.hydro_buoy = p.hydro_buoy;
    K.t_limiter = p.t_limiter;
    K.cell_hold = p.cell_hold;
    K.rad_on = (p.rad_coupling != 0.0 && p.cp_mix > 0.0);
    K.precip_on = (p.precip_coupling != 0.0 && p.r_mix > 0.0 && p.cp_mix > 0.0);
    K.tmf_on = (p.thermal_massflux != 0.0);
    K.divu_on = (p.species_divu != 0.0);
    K.press_incr = (p.press_incr != 0 && p.press_src != 0);
    K.press_src = p.press_src;
    K.rigid_lid = p.rigid_lid;
    K.press_wall = p.press_wall;
    K.dr = g.dr;
    K.inv_2dr = 1.0 / (2.0 * g.dr);
    K.inv_2dthe = 1.0 / (2.0 * g.dthe);
    K.inv_2dphi = 1.0 / (2.0 * g.dphi);
    K.inv_dr2 = 1.0 / (g.dr * g.dr);
    K.inv_dthe2 = 1.0 / (g.dthe * g.dthe);
    K.inv_dphi2 = 1.0 / (g.dphi * g.dphi);
    K.coeff_energy_p = p.u_0 * p.u_0 / (p.cp_mix * p.t_ref);
    K.to_nd = 1.0 / (p.r_mix * p.u_0 * p.u_0 * 1.0e-5);
    K.r_mix = p.r_mix;
    K.rR = p.r_mix * p.R_mix;
    K.buoy_c = p.g / (K.rR * p.t_ref);
    K.t_ref = p.t_ref;
    K.g = p.g;
    const double L_m = p.L_atm * 1.0e3;
    const double nd_buoy = p.nd_buoy ? 1.0e5 * L_m / (p.u_0 * p.u_0) : 1.0;
    K.kbuoy = -nd_buoy * p.buoy_scale * p.buoyancy;
    K.legacy_buoy = p.buoyancy * p.g;
    K.inv_re = 1.0 / p.re;
    K.inv_re_pr = 1.0 / (p.re * p.pr);
    K.inv_sc_re_ch4 = 1.0 / (p.sc_ch4 * p.re);
    K.inv_sc_re_h2o = 1.0 / (p.sc_h2o * p.re);
    K.inv_sc_re_h2s = 1.0 / (p.sc_h2s * p.re);
    K.inv_sc_re_nh3 = 1.0 / (p.sc_nh3 * p.re);
    K.inv_sc_re_nh4sh = 1.0 / (p.sc_nh4sh * p.re);
    K.inv_sig_k = 1.0 / 0.85;
    K.inv_sig_w = 1.0 / 0.5;
    K.turb_coupling = p.turb_coupling;
    K.inv_pr_t = 1.0 / 0.9;
    K.Coriolis = p.Coriolis;
    K.centrifugal = p.centrifugal;
    K.chem = p.chemical_reaction;
    K.metric_on = p.metric_split ? 0.0 : 1.0;
    K.cor_rad_on = p.coriolis_split ? 0.0 : 1.0;
    K.rad_coupling = p.rad_coupling;
    K.rad_num = L_m;
    K.rad_den_c = p.cp_mix * p.u_0 * p.t_ref;
    K.precip_coupling = p.precip_coupling;
    K.precip_num = L_m;
    K.precip_den = 1.0 / (p.r_mix * p.cp_mix * p.u_0 * p.t_ref);
    K.tmf_chem = p.thermal_massflux * p.chemical_reaction;
    K.species_divu = p.species_divu;
    K.tke_max = 1000.0 / (p.u_0 * p.u_0);
    K.dis_min = 1.0e-10;
    K.dt = p.dt;
    K.pdyn_cap = p.pdyn_cap;
    K.c43 = 4.0 / 3.0;
    K.c13 = 1.0 / 3.0;
}

// Per-column geometry (RungeKutta_Sat_Turb.cpp:129-142, 223-243; PressureSolver.h:156-162, 255-259, 326-353)
void build_geometry(atsat_dyn* h, const double* vbar0, const double* ubar0) {
    const atsat_dyn_params& p = h->p;
    const atsat_dyn_grid& g = h->g;
    const int im = g.im, jm = g.jm;
    h->geo_h.assign((size_t)im * jm, ColGeo{});
    const double L_m = p.L_atm * 1.0e3;
    const double nd_cor = p.nd_cor ? L_m / p.u_0 : 1.0;
    const double nd_cent = p.nd_cent ? L_m * L_m / (p.u_0 * p.u_0) : 1.0;
    const double inv_dr2 = 1.0 / (g.dr * g.dr), inv_dthe2 = 1.0 / (g.dthe * g.dthe);
    const double inv_dphi2 = 1.0 / (g.dphi * g.dphi);
    for (int i = 0; i < im; i++) {
        for (int j = 0; j < jm; j++) {
            ColGeo& c = h->geo_h[(size_t)i * jm + j];
            double st = std::sin(h->the_z[j]);
            if (st < p.sinthe_min) st = p.sinthe_min;
            const double ct = std::cos(h->the_z[j]);
            const double rm = metric_radius(p, h->rad_z[i]);
            const double rm2 = rm * rm;
            const double sinthe2 = st * st;
            c.rm = rm;
            c.inv_rm = 1.0 / rm;
            c.inv_rm2 = 1.0 / rm2;
            c.inv_rmsinthe = 1.0 / (rm * st);
            c.inv_rm2sinthe = c.inv_rm2 / st;
            c.inv_rm2sinthe2 = c.inv_rm2 / sinthe2;
            c.costhe_inv_rm2sinthe = ct * c.inv_rm2sinthe;
            c.cotanthe = ct / st;
            c.costhe = ct;
            c.two_inv_rm = 2.0 * c.inv_rm;
            c.v_metric = (1.0 + ct / sinthe2) * c.inv_rm2;
            c.exp_rm = 1.0;
            c.exp_2_rm = 1.0;
            const double s_true = std::sqrt(std::max(0.0, 1.0 - ct * ct));
            c.sinthe_true = s_true;
            c.cor_rad = nd_cor * -2.0 * p.omega * s_true;
            c.cor_the = nd_cor * -2.0 * p.omega * ct;
            c.cor_phi = nd_cor * +2.0 * p.omega;
            c.cent_rad = nd_cent * p.omega * p.omega * rm * s_true * s_true;
            c.cent_the = nd_cent * p.omega * p.omega * rm * s_true * ct;
            const bool hold = p.cell_hold && vbar0 && ubar0;
            c.vbar0 = hold ? vbar0[(size_t)i * jm + j] : 0.0;
            c.ubar0 = hold ? ubar0[(size_t)i * jm + j] : 0.0;
            // pressure solver: its own sine table with the exact-zero guard
            double sp = std::sin(h->the_z[j]);
            if (sp < p.sinthe_min) sp = p.sinthe_min;
            if (sp == 0.0) sp = 1.0e-5;
            const double inv_rm2 = 1.0 / rm2;
            const double inv_rm2sinthe2 = inv_rm2 / (sp * sp);
            c.p_num1 = 1.0 * inv_dr2;
            c.p_num2 = inv_rm2 * inv_dthe2;
            c.p_num3 = inv_rm2sinthe2 * inv_dphi2;
            c.p_den = 2.0 * c.p_num1 + 2.0 * c.p_num2 + 2.0 * c.p_num3;
            c.lc_num1 = 1.0 * 1.0 * inv_dr2;
            c.lc_num2 = inv_dthe2 / (rm * rm);
            c.lc_num3 = inv_dphi2 / (rm * rm * sp * sp);
            c.p_exp_rm = 1.0;
            c.p_inv_rm = 1.0 / rm;
            c.p_inv_rmsinthe = 1.0 / (rm * sp);
            c.p_pad_cot_rm = c.cotanthe * c.inv_rm;
            c.src_r = c.p_exp_rm / (2.0 * g.dr);
            c.src_the = c.p_inv_rm / (2.0 * g.dthe);
            c.src_phi = c.p_inv_rmsinthe / (2.0 * g.dphi);
            c.p_inv_den = 1.0 / c.p_den;
            {
                const double i2dr = 1.0 / (2.0 * g.dr), i2dthe = 1.0 / (2.0 * g.dthe), i2dphi = 1.0 / (2.0 * g.dphi);
                c.t_the = i2dthe * c.inv_rm;
                c.t_phi = i2dphi * c.inv_rmsinthe;
                c.d_r1 = c.two_inv_rm * i2dr;
                c.d_t2 = c.inv_rm2 * inv_dthe2;
                c.d_t1 = c.costhe_inv_rm2sinthe * i2dthe;
                c.d_p2 = c.inv_rm2sinthe2 * inv_dphi2;
                c.x_v1 = 2.0 * c.inv_rm2 * i2dthe;
                c.x_v2 = 2.0 * c.costhe * c.inv_rm2sinthe2 * i2dphi;
                c.x_w1 = 2.0 * c.inv_rm2sinthe * i2dphi;
            }
        }
    }
}

// FP32 constants of the mixed stage kernel, formed from the FP64 ones.
void build_mixed_constants(atsat_dyn* h) {
    const KConst& K = h->kc;
    const atsat_dyn_params& p = h->p;
    MixedConstF& F = h->kf;
    F.im = K.im; F.jm = K.jm; F.km = K.km; F.kp = K.kp; F.plane = K.plane;
    F.metric_split = K.metric_split; F.hydro_buoy = K.hydro_buoy; F.turb = K.turb; F.rad_on = K.rad_on;
    F.precip_on = K.precip_on; F.tmf_on = K.tmf_on; F.divu_on = K.divu_on;
    F.fsz_over_int = K.fsz >= (int64_t)0x7FFFFFFF ? 1 : 0;
    F.inv_2dr = (float)K.inv_2dr; F.inv_2dthe = (float)K.inv_2dthe; F.inv_2dphi = (float)K.inv_2dphi;
    F.inv_dr2 = (float)K.inv_dr2; F.inv_dthe2 = (float)K.inv_dthe2; F.inv_dphi2 = (float)K.inv_dphi2;
    F.coeff_energy_p = (float)K.coeff_energy_p; F.inv_re = (float)K.inv_re; F.inv_re_pr = (float)K.inv_re_pr;
    F.inv_sc_re_ch4 = (float)K.inv_sc_re_ch4; F.inv_sc_re_h2o = (float)K.inv_sc_re_h2o;
    F.inv_sc_re_h2s = (float)K.inv_sc_re_h2s; F.inv_sc_re_nh3 = (float)K.inv_sc_re_nh3;
    F.inv_sc_re_nh4sh = (float)K.inv_sc_re_nh4sh;
    F.inv_sig_k = (float)K.inv_sig_k; F.inv_sig_w = (float)K.inv_sig_w;
    F.turb_coupling = (float)K.turb_coupling; F.inv_pr_t = (float)K.inv_pr_t;
    F.chem = (float)K.chem; F.precip_coupling = (float)K.precip_coupling;
    F.precip_factor = (float)(K.precip_coupling * K.precip_num * K.precip_den);
    F.rad_factor = (float)(K.rad_coupling * K.rad_num / K.rad_den_c);
    F.r_mix = (float)K.r_mix;
    F.tke_max = (float)K.tke_max; F.dis_min = (float)K.dis_min;
    F.species_divu = (float)K.species_divu; F.tmf_chem = (float)K.tmf_chem;
    F.metric_on = (float)K.metric_on; F.cor_rad_on = (float)K.cor_rad_on;
    F.kb = p.buoy_legacy ? 1.0f : (float)K.kbuoy;
    F.bref_scale = p.buoy_legacy ? 0.0f : 1.0f;
    F.tke_max_d = K.tke_max; F.dis_min_d = K.dis_min;
}

cudaError_t upload_geof(atsat_dyn* h) {
    const atsat_dyn_params& p = h->p;
    std::vector<ColGeoF> gf(h->geo_h.size());
    for (size_t n = 0; n < gf.size(); n++) {
        const ColGeo& c = h->geo_h[n];
        ColGeoF& f = gf[n];
        f.inv_rm = (float)c.inv_rm; f.inv_rm2 = (float)c.inv_rm2; f.inv_rmsinthe = (float)c.inv_rmsinthe;
        f.inv_rm2sinthe = (float)c.inv_rm2sinthe; f.inv_rm2sinthe2 = (float)c.inv_rm2sinthe2;
        f.costhe_inv_rm2sinthe = (float)c.costhe_inv_rm2sinthe; f.cotanthe = (float)c.cotanthe;
        f.costhe = (float)c.costhe; f.two_inv_rm = (float)c.two_inv_rm; f.v_metric = (float)c.v_metric;
        f.sinthe_true = (float)c.sinthe_true;
        f.cor_the_c = (float)(p.Coriolis * c.cor_the);
        f.cor_phi_c = (float)(p.Coriolis * c.cor_phi);
        f.cor_rad_c = (float)(p.Coriolis * c.cor_rad);
        f.vbar0 = (float)c.vbar0; f.ubar0 = (float)c.ubar0;
    }
    // the prepare kernel's column products, in FP64 (and the two pure scalings in FP32)
    const KConst& K = h->kc;
    std::vector<PrepGeo> pg(h->geo_h.size());
    for (size_t n = 0; n < pg.size(); n++) {
        const ColGeo& c = h->geo_h[n];
        PrepGeo& g = pg[n];
        g.s_the = K.inv_2dthe * c.inv_rm;
        g.cot_rm = c.p_pad_cot_rm;
        g.cor_the_c = K.Coriolis * c.cor_the;
        g.cent_the_c = K.centrifugal * c.cent_the;
        g.cent_rad_c = K.centrifugal * c.cent_rad;
        g.cor_rad_c = K.cor_rad_on * K.Coriolis * c.cor_rad;
        g.metric_inv_rm = K.metric_on * c.inv_rm;
        g.s_the_f = (float)(K.inv_2dthe * c.inv_rm);
        g.s_phi_f = (float)(K.inv_2dphi * c.inv_rmsinthe);
    }
    cudaError_t e = cudaMemcpyAsync(h->geof, gf.data(), sizeof(ColGeoF) * gf.size(), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(h->pgeo, pg.data(), sizeof(PrepGeo) * pg.size(), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(h->stream);
}

// The tiled stage kernel's tensor maps: slab32 as a 4-D FP32 tensor (k, j, i, array) with the strides
// of the device layout; boxes of TILE_BX x TILE_BY x TILE_BZ (halo box) and TILE_SEAM_X x TILE_J x
// TILE_I (seam column). Out-of-range parts of a box read as zero. false when the driver offers no
// encoder or rejects the maps; the direct kernel runs then.
bool make_tile_maps(atsat_dyn* h) {
    using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult qr = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr) != cudaSuccess ||
        qr != cudaDriverEntryPointSuccess || fn == nullptr) {
        cudaGetLastError();
        return false;
    }
    const KConst& K = h->kc;
    if ((reinterpret_cast<uintptr_t>(h->slab32) & 15u) != 0) return false;
    // the innermost extent is km, not the padded row kp: the padding columns are never a cell or a stencil
    // neighbour (the east neighbour of km-2 is the periodic seam k = 0), so boxes of the last k-tile read
    // only the row's km values and the tensor copy fills the rest of the box with zeros
    const cuuint64_t dims[4] = {(cuuint64_t)K.km, (cuuint64_t)K.jm, (cuuint64_t)K.im, (cuuint64_t)h->n32};
    const cuuint64_t strides[3] = {(cuuint64_t)K.kp * 4, (cuuint64_t)K.plane * 4, (cuuint64_t)K.fsz * 4};
    const cuuint32_t box_main[4] = {TILE_BX, TILE_BY, TILE_BZ, 1};
    const cuuint32_t box_seam[4] = {TILE_SEAM_X, TILE_J, TILE_I, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const Encode enc = reinterpret_cast<Encode>(fn);
    const CUresult r1 = enc(reinterpret_cast<CUtensorMap*>(h->maps.main), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->slab32,
                            dims, strides, box_main, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const CUresult r2 = enc(reinterpret_cast<CUtensorMap*>(h->maps.seam), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->slab32,
                            dims, strides, box_seam, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const cuuint32_t box_main4[4] = {TILE_BX, TILE_BY, TTILE_BZ, 1};
    const cuuint32_t box_seam4[4] = {TILE_SEAM_X, TILE_J, TTILE_I, 1};
    const CUresult r3 = enc(reinterpret_cast<CUtensorMap*>(h->maps.main4), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->slab32,
                            dims, strides, box_main4, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const CUresult r4 = enc(reinterpret_cast<CUtensorMap*>(h->maps.seam4), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->slab32,
                            dims, strides, box_seam4, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const cuuint32_t box_pt4[4] = {TILE_K, TILE_J, TTILE_I, 1};
    const CUresult r5 = enc(reinterpret_cast<CUtensorMap*>(h->maps.pt4), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->slab32,
                            dims, strides, box_pt4, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const cuuint32_t box_pt2[4] = {TILE_K, TILE_J, TILE_I, 1};
    const CUresult r6 = enc(reinterpret_cast<CUtensorMap*>(h->maps.pt2), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h->slab32,
                            dims, strides, box_pt2, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    // the radial march's planes: one level deep
    const cuuint32_t box_plane1[4] = {TILE_BX, TILE_BY, 1, 1};
    const cuuint32_t box_seam1[4] = {TILE_SEAM_X, TILE_J, 1, 1};
    const cuuint32_t box_pt1[4] = {TILE_K, TILE_J, 1, 1};
    const CUresult r7 = enc(reinterpret_cast<CUtensorMap*>(h->maps.plane1), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                            h->slab32, dims, strides, box_plane1, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const CUresult r8 = enc(reinterpret_cast<CUtensorMap*>(h->maps.seam1), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                            h->slab32, dims, strides, box_seam1, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    const CUresult r9 = enc(reinterpret_cast<CUtensorMap*>(h->maps.pt1), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                            h->slab32, dims, strides, box_pt1, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r1 == CUDA_SUCCESS && r2 == CUDA_SUCCESS && r3 == CUDA_SUCCESS && r4 == CUDA_SUCCESS && r5 == CUDA_SUCCESS &&
           r6 == CUDA_SUCCESS && r7 == CUDA_SUCCESS && r8 == CUDA_SUCCESS && r9 == CUDA_SUCCESS;
}

bool valid_field(int f) { return f >= 0 && f < ATSAT_NFIELDS; }

// FP32 copies kept for the mixed path: rho_mix and the point inputs nue .. thermalmassflux.
int conv_slot(int fid) {
    if (fid == ATSAT_F_RHO_MIX) return 0;
    if (fid >= ATSAT_F_NUE && fid <= ATSAT_F_THERMALMASSFLUX) return 1 + (fid - ATSAT_F_NUE);
    return -1;
}
int conv_field(int slot) { return slot == 0 ? ATSAT_F_RHO_MIX : ATSAT_F_NUE + slot - 1; }

void mark_dirty(atsat_dyn* h, int fid) {
    const int s = conv_slot(fid);
    if (s >= 0) h->conv_dirty[s] = true;
}

// Contiguous host arrays hold im*jm*km doubles per field while the device rows are kp doubles long. A
// pitched 2-D copy of 2.9 KB rows runs far below the link, so every field goes as one contiguous copy into a
// device staging buffer and a kernel moves it to (or from) the pitched layout. Two buffers alternate: the
// copy stream carries the transfers, the handle stream the re-pitch kernels, and events order each buffer's
// producer before its consumer and its consumer before the buffer's next producer, so the transfer of one
// field overlaps the re-pitch of the one before.
void stage_pipe_free(atsat_dyn* h) {
    if (h->cstream) cudaStreamSynchronize(h->cstream);
    for (int b = 0; b < 2; b++) {
        if (h->dstage[b]) cudaFree(h->dstage[b]);
        if (h->ev_ready[b]) cudaEventDestroy(h->ev_ready[b]);
        if (h->ev_free[b]) cudaEventDestroy(h->ev_free[b]);
        h->dstage[b] = nullptr;
        h->ev_ready[b] = h->ev_free[b] = nullptr;
    }
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->cstream) cudaStreamDestroy(h->cstream);
    h->ev_join = nullptr;
    h->cstream = nullptr;
}

// All or nothing: the copy stream exists only when both buffers and all events do.
int stage_pipe_create(atsat_dyn* h) {
    CK(h, cudaSetDevice(h->device));
    const size_t bytes = (size_t)h->kc.im * h->kc.jm * h->kc.km * 8;
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMalloc(&h->dstage[b], bytes);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_ready[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_free[b], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        stage_pipe_free(h);
        cudaGetLastError();
        return fail(h, ATSAT_DYN_E_NOMEM, "device staging: %s", cudaGetErrorString(e));
    }
    h->stage_next = 0;
    return ATSAT_DYN_OK;
}

int stage_in(atsat_dyn* h, double* dst, const double* host) {
    const KConst& K = h->kc;
    const int b = h->stage_next;
    h->stage_next ^= 1;
    CK(h, cudaStreamWaitEvent(h->cstream, h->ev_free[b], 0));
    CK(h, cudaMemcpyAsync(h->dstage[b], host, (size_t)K.im * K.jm * K.km * 8, cudaMemcpyHostToDevice, h->cstream));
    CK(h, cudaEventRecord(h->ev_ready[b], h->cstream));
    CK(h, cudaStreamWaitEvent(h->stream, h->ev_ready[b], 0));
    CK(h, launch_repitch(dst, K.kp, h->dstage[b], K.km, K.km, (int64_t)K.im * K.jm, h->stream));
    h->launches += 1;
    CK(h, cudaEventRecord(h->ev_free[b], h->stream));
    return ATSAT_DYN_OK;
}

int stage_out(atsat_dyn* h, double* host, const double* src) {
    const KConst& K = h->kc;
    const int b = h->stage_next;
    h->stage_next ^= 1;
    CK(h, cudaStreamWaitEvent(h->stream, h->ev_free[b], 0));
    CK(h, launch_repitch(h->dstage[b], K.km, src, K.kp, K.km, (int64_t)K.im * K.jm, h->stream));
    h->launches += 1;
    CK(h, cudaEventRecord(h->ev_ready[b], h->stream));
    CK(h, cudaStreamWaitEvent(h->cstream, h->ev_ready[b], 0));
    CK(h, cudaMemcpyAsync(host, h->dstage[b], (size_t)K.im * K.jm * K.km * 8, cudaMemcpyDeviceToHost, h->cstream));
    CK(h, cudaEventRecord(h->ev_free[b], h->cstream));
    return ATSAT_DYN_OK;
}

// The handle stream waits for everything queued on the copy stream, so one synchronisation of it covers both.
int stage_join(atsat_dyn* h) {
    if (!h->cstream) return ATSAT_DYN_OK;
    CK(h, cudaEventRecord(h->ev_join, h->cstream));
    CK(h, cudaStreamWaitEvent(h->stream, h->ev_join, 0));
    return ATSAT_DYN_OK;
}

int upload_one(atsat_dyn* h, int fid) {
    const KConst& K = h->kc;
    mark_dirty(h, fid);
    const int im = K.im, jm = K.jm, km = K.km, kp = K.kp;
    if (h->bind_kind[fid] == BIND_ARRAY) {
        const size_t n = (size_t)im * jm * km;
        if (kp == km) {
            CK(h, cudaMemcpyAsync(h->f[fid], h->bind_base[fid], n * 8, cudaMemcpyHostToDevice, h->stream));
        } else {
            int rc = stage_in(h, h->f[fid], h->bind_base[fid]);
            if (rc) return rc;
        }
    } else if (h->bind_kind[fid] == BIND_ROWS) {
        const int b = h->pin_next;
        h->pin_next ^= 1;
        CK(h, cudaEventSynchronize(h->ev_pin[b]));  // the previous copy out of this buffer has finished
        double* const* rows = h->bind_rows[fid].data();
        double* st = h->pinned[b];
        const int nrows = im * jm;
#pragma omp parallel for schedule(static)
        for (int r = 0; r < nrows; r++) memcpy(st + (size_t)r * kp, rows[r], (size_t)km * 8);
        CK(h, cudaMemcpyAsync(h->f[fid], st, (size_t)K.fsz * 8, cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaEventRecord(h->ev_pin[b], h->stream));
    } else {
        return fail(h, ATSAT_DYN_E_UNBOUND, "field %d has no host binding", fid);
    }
    return ATSAT_DYN_OK;
}

// Unpacks the field whose device->host copy was queued last, once that copy has landed.
int rows_flush(atsat_dyn* h) {
    const int fid = h->rows_pending;
    if (fid < 0) return ATSAT_DYN_OK;
    h->rows_pending = -1;
    const KConst& K = h->kc;
    const int b = h->rows_pending_buf;
    CK(h, cudaEventSynchronize(h->ev_pin[b]));
    double* const* rows = h->bind_rows[fid].data();
    const double* st = h->pinned[b];
    const int nrows = K.im * K.jm, km = K.km, kp = K.kp;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < nrows; r++) memcpy(rows[r], st + (size_t)r * kp, (size_t)km * 8);
    return ATSAT_DYN_OK;
}

int download_one(atsat_dyn* h, int fid) {
    const KConst& K = h->kc;
    const int im = K.im, jm = K.jm, km = K.km, kp = K.kp;
    if (h->bind_kind[fid] == BIND_ARRAY) {
        const size_t n = (size_t)im * jm * km;
        if (kp == km) {
            CK(h, cudaMemcpyAsync(h->bind_base[fid], h->f[fid], n * 8, cudaMemcpyDeviceToHost, h->stream));
        } else {
            int rc = stage_out(h, h->bind_base[fid], h->f[fid]);
            if (rc) return rc;
        }
    } else if (h->bind_kind[fid] == BIND_ROWS) {
        // the buffer was last read by the unpack two fields ago, which the flush below has completed
        const int b = h->pin_next;
        h->pin_next ^= 1;
        CK(h, cudaMemcpyAsync(h->pinned[b], h->f[fid], (size_t)K.fsz * 8, cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaEventRecord(h->ev_pin[b], h->stream));
        int rc = rows_flush(h);
        if (rc) return rc;
        h->rows_pending = fid;
        h->rows_pending_buf = b;
    } else {
        return fail(h, ATSAT_DYN_E_UNBOUND, "field %d has no host binding", fid);
    }
    return ATSAT_DYN_OK;
}

// The copy-engine path's resources for a binding: pinned staging for ragged rows, the device staging
// pipeline for contiguous arrays whose rows the device pads.
int staging_for(atsat_dyn* h, int fid) {
    if (h->bind_kind[fid] == BIND_ROWS && !h->ev_pin[1]) {
        CK(h, cudaSetDevice(h->device));
        cudaError_t e = cudaSuccess;
        for (int b = 0; b < 2 && e == cudaSuccess; b++) {
            if (!h->pinned[b]) e = cudaHostAlloc(&h->pinned[b], (size_t)h->kc.fsz * 8, cudaHostAllocDefault);
            if (e == cudaSuccess && !h->ev_pin[b]) e = cudaEventCreateWithFlags(&h->ev_pin[b], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(h, ATSAT_DYN_E_NOMEM, "pinned staging: %s", cudaGetErrorString(e));
        }
    }
    if (h->bind_kind[fid] == BIND_ARRAY && !h->cstream && h->kc.kp != h->kc.km) return stage_pipe_create(h);
    return ATSAT_DYN_OK;
}

// Chooses the path of field fid's binding: the SMs in place when selected (a ragged binding's row table
// then goes to the device once, here), else the copy engines.
int route_binding(atsat_dyn* h, int fid) {
    h->direct[fid] = false;
    if (h->bind_kind[fid] == BIND_NONE) return ATSAT_DYN_OK;
    bool aligned = (reinterpret_cast<uintptr_t>(h->bind_base[fid]) & 7u) == 0;   // whole doubles only
    for (double* r : h->bind_rows[fid]) aligned = aligned && (reinterpret_cast<uintptr_t>(r) & 7u) == 0;
    if (!h->host_direct || !aligned) return staging_for(h, fid);
    if (h->bind_kind[fid] == BIND_ROWS) {
        const size_t n = h->bind_rows[fid].size();
        CK(h, cudaSetDevice(h->device));
        if (!h->dev_rows[fid]) {
            const cudaError_t e = cudaMalloc(&h->dev_rows[fid], n * sizeof(double*));
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(h, ATSAT_DYN_E_NOMEM, "row table: %s", cudaGetErrorString(e));
            }
        }
        // a transfer queued earlier (asynchronous mode) may still read the old table
        CK(h, cudaStreamSynchronize(h->stream));
        CK(h, cudaMemcpy(h->dev_rows[fid], h->bind_rows[fid].data(), n * sizeof(double*), cudaMemcpyHostToDevice));
    }
    h->direct[fid] = true;
    return ATSAT_DYN_OK;
}

int batch_flush(atsat_dyn* h, HostBatch& b, int to_device) {
    if (b.n == 0) return ATSAT_DYN_OK;
    const KConst& K = h->kc;
    CK(h, launch_host_transfer(b, to_device, (int64_t)K.im * K.jm, K.km, K.kp, h->stream));
    h->launches += 1;
    b.n = 0;
    return ATSAT_DYN_OK;
}

int batch_add(atsat_dyn* h, HostBatch& b, int fid, int to_device) {
    if (b.n == HOST_BATCH_MAX) {
        int rc = batch_flush(h, b, to_device);
        if (rc) return rc;
    }
    HostField& f = b.f[b.n++];
    f.base = h->bind_kind[fid] == BIND_ARRAY ? h->bind_base[fid] : nullptr;
    f.rows = h->bind_kind[fid] == BIND_ROWS ? h->dev_rows[fid] : nullptr;
    f.dev = h->f[fid];
    f.dev32 = nullptr;
    const int slot = conv_slot(fid);
    if (to_device && slot >= 0 && h->slab32) {
        // the mixed path's FP32 copy is written in the same pass (d2f: the hardware's rounding) and is current
        f.dev32 = h->conv32[slot];
        h->conv_dirty[slot] = false;
    }
    return ATSAT_DYN_OK;
}

// The end of an entry point: launch errors always; in the asynchronous mode nothing else unless the call
// hands a device result to the host (host_result), else the wait for the stream and the device status word.
int finish(atsat_dyn* h, bool host_result = false) {
    CK(h, cudaGetLastError());
    if (h->async && !host_result) return ATSAT_DYN_OK;
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->dev_err && h->tile_ok) {
        unsigned int v = 0;
        CK(h, cudaMemcpy(&v, h->dev_err, sizeof(v), cudaMemcpyDeviceToHost));
        if (v) {
            CK(h, cudaMemset(h->dev_err, 0, sizeof(v)));
            h->timeouts++;
            return fail(h, ATSAT_DYN_E_TIMEOUT, "tiled stage kernel: device status 0x%x (1 producer wait, 2 consumer "
                        "wait, 4 plan mismatch, 8 shared-memory alignment)", v);
        }
    }
    return ATSAT_DYN_OK;
}

StageIO<double> make_io(atsat_dyn* h, double* const* in, double* const* out) {
    StageIO<double> io{};
    for (int q = 0; q < NPROG; q++) {
        io.in[q] = in[q];
        io.out[q] = out ? out[q] : nullptr;
        io.yn[q] = h->f[ATSAT_F_N_BASE + q];
        io.acc[q] = h->acc[q];
        io.rhs[q] = h->f[ATSAT_F_RHS_BASE + q];
    }
    io.p_dyn = h->f[ATSAT_F_P_DYN];
    io.p_stat = h->f[ATSAT_F_P_STAT];
    io.p_metric = h->f[ATSAT_F_P_METRIC];
    io.rho_mix = h->f[ATSAT_F_RHO_MIX];
    io.nue = h->f[ATSAT_F_NUE];
    io.q_precip = h->f[ATSAT_F_Q_PRECIP];
    io.q_rad = h->f[ATSAT_F_Q_RAD];
    io.tke_source = h->f[ATSAT_F_TKE_SOURCE];
    io.dis_source = h->f[ATSAT_F_DIS_SOURCE];
    for (int s = 0; s < 9; s++) io.s_precip[s] = h->f[ATSAT_F_S_PRECIP_H2O + s];
    io.massflux_h2s = h->f[ATSAT_F_MASSFLUX_H2S];
    io.massflux_nh3 = h->f[ATSAT_F_MASSFLUX_NH3];
    io.massflux_nh4sh = h->f[ATSAT_F_MASSFLUX_NH4SH];
    io.fluxlim_nh4sh = h->f[ATSAT_F_FLUXLIM_NH4SH];
    io.thermalmassflux = h->f[ATSAT_F_THERMALMASSFLUX];
    io.aux[0] = h->f[ATSAT_F_AUX_U];
    io.aux[1] = h->f[ATSAT_F_AUX_V];
    io.aux[2] = h->f[ATSAT_F_AUX_W];
    io.buoy = h->buoy;
    io.geo = h->geo;
    return io;
}

int do_level_mean(atsat_dyn* h) {
    Timed t(h, ATSAT_K_LEVEL_MEAN);
    CK(h, launch_level_mean(h->kc, h->f[ATSAT_F_T], h->f[ATSAT_F_P_STAT], h->sin_j, h->partial, h->buoy, h->stream));
    h->launches += 2;
    return ATSAT_DYN_OK;
}

int do_metric(atsat_dyn* h) {
    Timed t(h, ATSAT_K_METRIC_SCAN);
    CK(h, launch_metric_scan(h->kc, h->f[ATSAT_F_V], h->f[ATSAT_F_W], h->rm_tab, h->cor_j,
                             h->has_pbaro ? h->p_baro : nullptr, h->f[ATSAT_F_P_METRIC], h->stream));
    h->launches += 1;
    return ATSAT_DYN_OK;
}

// the start of a step: the buoyancy level mean and, where metric_split is on, the metric pressure. Both
// read y_n only and are latency-bound scans (GB300's FP64 pipe sets their pace, not HBM), so the metric scan
// runs on a second stream beside the level mean, forked from and joined back into the handle's stream by
// events (CUDA-graph capture records the fork and the join).
int do_level_metric(atsat_dyn* h) {
    if (!h->p.metric_split) return do_level_mean(h);
    if (!h->astream) {
        CK(h, cudaStreamCreateWithFlags(&h->astream, cudaStreamNonBlocking));
        CK(h, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
        CK(h, cudaEventCreateWithFlags(&h->ev_ajoin, cudaEventDisableTiming));
    }
    Timed t(h, ATSAT_K_LEVEL_MEAN);
    CK(h, cudaEventRecord(h->ev_fork, h->stream));
    CK(h, cudaStreamWaitEvent(h->astream, h->ev_fork, 0));
    CK(h, launch_metric_scan(h->kc, h->f[ATSAT_F_V], h->f[ATSAT_F_W], h->rm_tab, h->cor_j,
                             h->has_pbaro ? h->p_baro : nullptr, h->f[ATSAT_F_P_METRIC], h->astream));
    CK(h, launch_level_mean(h->kc, h->f[ATSAT_F_T], h->f[ATSAT_F_P_STAT], h->sin_j, h->partial, h->buoy, h->stream));
    CK(h, cudaEventRecord(h->ev_ajoin, h->astream));
    CK(h, cudaStreamWaitEvent(h->stream, h->ev_ajoin, 0));
    h->launches += 3;
    return ATSAT_DYN_OK;
}

int enqueue_rk4_mixed(atsat_dyn* h, bool resident);

int enqueue_rk4(atsat_dyn* h, bool resident = false) {
    if (h->p.precision == ATSAT_DYN_MIXED) return enqueue_rk4_mixed(h, resident);
    int rc;
    if ((rc = do_level_metric(h))) return rc;
    double* L[NPROG];
    double* S[NPROG];
    for (int q = 0; q < NPROG; q++) { L[q] = h->f[q]; S[q] = h->stage[q]; }
    const double dt = h->p.dt;
    for (int stage = 0; stage < 4; stage++) {
        StageParams sp{};
        sp.stage = stage;
        sp.write_all_rhs = h->write_all_rhs;
        sp.c_in = (stage == 0 || stage == 1) ? 0.5 * dt : (stage == 2 ? dt : 0.0);
        sp.wgt = (stage == 0 || stage == 3) ? 1.0 : 2.0;
        sp.sixth_dt = dt / 6.0;
        double* const* in = (stage & 1) ? S : L;
        double* const* out = (stage & 1) ? L : S;
        StageIO<double> io = make_io(h, in, out);
        Timed t(h, ATSAT_K_RK_STAGE);
        CK(h, launch_rk_stage_fp64(h->kc, io, sp, stage == 3 ? MODE_FINAL : MODE_STAGE, h->stream));
        h->launches += 1;
    }
    return ATSAT_DYN_OK;
}

MixedIO make_mixed_io(atsat_dyn* h, float* const* dl_in, float* const* dl_out, double* const* out64) {
    MixedIO io{};
    for (int q = 0; q < NPROG; q++) {
        io.yn64[q] = h->f[ATSAT_F_N_BASE + q];
        io.yn32[q] = h->yn32[q];
        io.dl_in[q] = dl_in ? dl_in[q] : nullptr;
        io.dl_out[q] = dl_out ? dl_out[q] : nullptr;
        io.dl1[q] = h->dlA[q];
        io.dl2[q] = h->dlB[q];
        io.out64[q] = out64 ? out64[q] : nullptr;
        io.out32[q] = nullptr;
        io.rhs[q] = h->f[ATSAT_F_RHS_BASE + q];
    }
    io.wlo = h->wlo;
    io.wlo_out = nullptr;
    io.acc_turb[0] = h->acc_turb[0];
    io.acc_turb[1] = h->acc_turb[1];
    for (int q = 0; q < NFZ; q++) io.fz[q] = h->fz[q];
    io.rho_mix = h->conv32[conv_slot(ATSAT_F_RHO_MIX)];
    io.nue = h->conv32[conv_slot(ATSAT_F_NUE)];
    io.q_precip = h->conv32[conv_slot(ATSAT_F_Q_PRECIP)];
    io.q_rad = h->conv32[conv_slot(ATSAT_F_Q_RAD)];
    io.tke_source = h->conv32[conv_slot(ATSAT_F_TKE_SOURCE)];
    io.dis_source = h->conv32[conv_slot(ATSAT_F_DIS_SOURCE)];
    for (int q = 0; q < 9; q++) io.s_precip[q] = h->conv32[conv_slot(ATSAT_F_S_PRECIP_H2O + q)];
    io.massflux_h2s = h->conv32[conv_slot(ATSAT_F_MASSFLUX_H2S)];
    io.massflux_nh3 = h->conv32[conv_slot(ATSAT_F_MASSFLUX_NH3)];
    io.massflux_nh4sh = h->conv32[conv_slot(ATSAT_F_MASSFLUX_NH4SH)];
    io.fluxlim_nh4sh = h->conv32[conv_slot(ATSAT_F_FLUXLIM_NH4SH)];
    io.thermalmassflux = h->conv32[conv_slot(ATSAT_F_THERMALMASSFLUX)];
    io.aux[0] = h->f[ATSAT_F_AUX_U];
    io.aux[1] = h->f[ATSAT_F_AUX_V];
    io.aux[2] = h->f[ATSAT_F_AUX_W];
    io.geof = h->geof;
    io.buoy = h->buoy;
    return io;
}

// Once per RK step: yn32 / wlo <- y_n (`base`) unless the resident copies are current, dl_0 <- live - y_n
// into all three increment buffers for the fields of dl0_mask (the cells no stage writes keep Y_s = live
// at every stage), the dirty FP32 input copies, and the frozen FP64 momentum terms.
int enqueue_mixed_prepare(atsat_dyn* h, double* const* base, uint32_t dl0_mask, bool resident) {
    MixedPrep pr{};
    pr.write_yn32 = resident ? 0 : 1;
    for (int q = 0; q < NPROG; q++) {
        const bool dl0 = (dl0_mask >> q) & 1u;
        pr.yn64[q] = base[q];
        pr.live64[q] = h->f[q];
        pr.yn32[q] = h->yn32[q];
        pr.yn32_b[q] = nullptr;
        pr.dl0[0][q] = dl0 ? h->dlC[q] : nullptr;
        pr.dl0[1][q] = dl0 ? h->dlA[q] : nullptr;
        pr.dl0[2][q] = dl0 ? h->dlB[q] : nullptr;
    }
    pr.any_dl0 = dl0_mask != 0;
    h->edges_dirty |= dl0_mask;
    pr.wlo = h->wlo;
    pr.wlo_b = nullptr;
    int n = 0;
    for (int sl = 0; sl < NCONV; sl++) {
        if (!h->conv_dirty[sl]) continue;
        pr.conv_src[n] = h->f[conv_field(sl)];
        pr.conv_dst[n] = h->conv32[sl];
        n++;
        h->conv_dirty[sl] = false;
    }
    pr.nconv = n;
    for (int q = 0; q < NFZ; q++) pr.fz[q] = h->fz[q];
    pr.p_dyn = h->f[ATSAT_F_P_DYN];
    pr.p_metric = h->f[ATSAT_F_P_METRIC];
    pr.p_stat = h->f[ATSAT_F_P_STAT];
    pr.rho_mix = h->f[ATSAT_F_RHO_MIX];
    pr.buoy = h->buoy;
    pr.pgeo = h->pgeo;
    pr.bnum = (h->p.buoy_legacy ? h->p.buoyancy * h->p.g : h->p.g) / (h->kc.rR * h->p.t_ref);
    pr.bnum_f = (float)pr.bnum;
    pr.cor_rad = h->kc.cor_rad_on != 0.0;
    pr.inv_2dr_f = (float)h->kc.inv_2dr;
    pr.dps_scale_f = (float)(h->kc.inv_2dr * h->kc.to_nd);
    pr.r_mix_f = (float)h->kc.r_mix;
    Timed t(h, ATSAT_K_PREPARE);
    CK(h, launch_mixed_prepare(h->kc, pr, h->stream));
    h->launches += 1;
    return ATSAT_DYN_OK;
}

int32_t arr_index(const atsat_dyn* h, const float* p) { return (int32_t)((p - h->slab32) / h->kc.fsz); }

// the arrays the tiled kernel streams, in the order it reads them: per field y_n, w's low word, the
// increment; tke and dis only with turbulence on
TilePlan make_plan(atsat_dyn* h, const MixedIO& io) {
    TilePlan pl{};
    pl.err = h->dev_err;
    pl.wait_limit = h->wait_limit;
    pl.arr_lo = arr_index(h, io.wlo);
    int n = 0;
    for (int q = 0; q < NPROG; q++) {
        pl.arr_yn[q] = arr_index(h, io.yn32[q]);
        pl.arr_dl[q] = io.dl_in[q] ? arr_index(h, io.dl_in[q]) : -1;
        if ((q == ATSAT_F_TKE || q == ATSAT_F_DIS) && !h->kc.turb) continue;
        pl.item[n++] = pl.arr_yn[q];
        if (q == ATSAT_F_W) pl.item[n++] = pl.arr_lo;
        if (io.dl_in[q]) pl.item[n++] = pl.arr_dl[q];
    }
    pl.n_items = n;
    return pl;
}

bool variant_available(const atsat_dyn* h, int v) {
    if (h->p.precision != ATSAT_DYN_MIXED) return v == ATSAT_DYN_STAGE_DIRECT;
    switch (v) {
        case ATSAT_DYN_STAGE_DIRECT: return true;
        case ATSAT_DYN_STAGE_TILED: return h->tile_ok;
        case ATSAT_DYN_STAGE_SPLIT:
        case ATSAT_DYN_STAGE_SPLIT3:
        case ATSAT_DYN_STAGE_SPLIT13: return !h->kc.divu_on;
        case ATSAT_DYN_STAGE_SPLIT_TILED:
        case ATSAT_DYN_STAGE_TILED2:
        case ATSAT_DYN_STAGE_MARCH: return !h->kc.divu_on && h->tile_ok && !h->kf.fsz_over_int;
        default: return false;
    }
}

int launches_per_stage(const atsat_dyn* h) { return h->variant >= ATSAT_DYN_STAGE_SPLIT ? 2 : 1; }

// The tracer kernel's stream, in the order its consumers read it: the winds' point values (u, [du], v,
// [dv], w, w's low word, [dw]) and nue; then per tracer field its y_n and increment halo boxes, its
// sources, the tke/dis running sum, and at the final stage dl_1 and dl_2.
TracerPlan make_plan_tracer(atsat_dyn* h, const MixedIO& io, int mode) {
    TracerPlan pl{};
    pl.err = h->dev_err;
    pl.wait_limit = h->wait_limit;
    pl.withhold = h->test_withhold;
    int n = 0;
    auto add = [&](const float* p, int kind) {
        if (n < TRACER_MAX_ITEMS) { pl.arr[n] = arr_index(h, p); pl.kind[n] = (unsigned char)kind; }
        n++;
    };
    const bool dl = io.dl_in[0] != nullptr;
    add(io.yn32[ATSAT_F_U], 1); if (dl) add(io.dl_in[ATSAT_F_U], 1);
    add(io.yn32[ATSAT_F_V], 1); if (dl) add(io.dl_in[ATSAT_F_V], 1);
    add(io.yn32[ATSAT_F_W], 1); add(io.wlo, 1); if (dl) add(io.dl_in[ATSAT_F_W], 1);
    add(io.nue, 1);
    for (int q = ATSAT_F_H2O; q < NPROG; q++) {
        const bool turb = q == ATSAT_F_TKE || q == ATSAT_F_DIS;
        if (turb && !h->kc.turb) continue;
        add(io.yn32[q], 0);
        if (dl) add(io.dl_in[q], 0);
        switch (q) {
            case ATSAT_F_H2O: add(io.s_precip[0], 1); break;
            case ATSAT_F_H2O_CLOUD: add(io.s_precip[1], 1); break;
            case ATSAT_F_H2O_ICE: add(io.s_precip[2], 1); break;
            case ATSAT_F_H2S: add(io.massflux_h2s, 1); break;
            case ATSAT_F_NH3: add(io.massflux_nh3, 1); add(io.s_precip[3], 1); break;
            case ATSAT_F_NH3_CLOUD: add(io.s_precip[4], 1); break;
            case ATSAT_F_NH3_ICE: add(io.s_precip[5], 1); break;
            case ATSAT_F_CH4: add(io.s_precip[6], 1); break;
            case ATSAT_F_CH4_CLOUD: add(io.s_precip[7], 1); break;
            case ATSAT_F_CH4_ICE: add(io.s_precip[8], 1); break;
            case ATSAT_F_NH4SH: add(io.fluxlim_nh4sh, 1); add(io.massflux_nh4sh, 1); break;
            case ATSAT_F_TKE: add(io.tke_source, 1); break;
            default: add(io.dis_source, 1); break;
        }
        if (turb) add(io.acc_turb[q - ATSAT_F_TKE], 1);
        else if (mode == MODE_FINAL) { add(io.dl1[q], 1); add(io.dl2[q], 1); }
    }
    pl.n_items = n;
    return pl;
}

// The momentum kernel's stream: nue; the halo boxes of u, v, w (with its low word) and t, y_n then the
// increment; then the frozen terms and inputs in the groups rhs_u, rhs_v, rhs_w and rhs_t use them.
TracerPlan make_plan_mom(atsat_dyn* h, const MixedIO& io) {
    TracerPlan pl{};
    pl.err = h->dev_err;
    pl.wait_limit = h->wait_limit;
    pl.withhold = h->test_withhold;
    int n = 0;
    auto add = [&](const float* p, int kind) {
        if (n < TRACER_MAX_ITEMS) { pl.arr[n] = arr_index(h, p); pl.kind[n] = (unsigned char)kind; }
        n++;
    };
    const bool dl = io.dl_in[0] != nullptr;
    add(io.nue, 1);
    add(io.yn32[ATSAT_F_U], 0); if (dl) add(io.dl_in[ATSAT_F_U], 0);
    add(io.yn32[ATSAT_F_V], 0); if (dl) add(io.dl_in[ATSAT_F_V], 0);
    add(io.yn32[ATSAT_F_W], 0); add(io.wlo, 0); if (dl) add(io.dl_in[ATSAT_F_W], 0);
    add(io.yn32[ATSAT_F_T], 0); if (dl) add(io.dl_in[ATSAT_F_T], 0);
    add(io.fz[FZ_DPR], 1); add(io.fz[FZ_GU], 1); add(io.fz[FZ_BAN], 1); add(io.fz[FZ_BPS], 1);
    add(io.fz[FZ_DPTH], 1); add(io.fz[FZ_GV], 1);
    add(io.fz[FZ_DPPH], 1); add(io.fz[FZ_GW], 1);
    add(io.fz[FZ_DPS], 1); add(io.rho_mix, 1); add(io.q_rad, 1); add(io.q_precip, 1); add(io.thermalmassflux, 1);
    pl.n_items = n;
    return pl;
}

// ---- the autotune cache ----
// One line per tuned configuration: "<im> <jm> <km> <knobs> <gpu> <version> <variant> <levels> <ms>", the
// GPU's name with blanks replaced by '_', the latest line of a key winning. knobs: bit 0 turbulence, 1
// radiation source, 2 precipitation source, 3 thermal mass flux (they change the kernels' streams).
constexpr int TUNE_VERSION = 1;     // raised whenever a stage kernel's speed changes materially

std::string tune_cache_path(const char* path) {
    if (path && path[0]) return path;
    const char* env = std::getenv("ATSAT_DYN_TUNE_CACHE");
    if (env) {
        if (!env[0] || !std::strcmp(env, "0") || !std::strcmp(env, "off")) return "";
        return env;
    }
    const char* xdg = std::getenv("XDG_CACHE_HOME");
    const char* home = std::getenv("HOME");
    std::string dir = (xdg && xdg[0]) ? std::string(xdg) : (home && home[0]) ? std::string(home) + "/.cache" : "";
    if (dir.empty()) return "";
    return dir + "/atsat_dyn/autotune.txt";
}

std::string tune_gpu_token(const char* gpu) {
    std::string t = gpu && gpu[0] ? gpu : "unknown";
    for (char& ch : t)
        if (ch == ' ' || ch == '\t' || ch == '\n') ch = '_';
    return t;
}

bool tune_get(const std::string& path, int im, int jm, int km, unsigned knobs, const std::string& gpu, int* variant,
              int* levels, double* ms) {
    if (path.empty()) return false;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    char line[512], g[256];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        int a, b, c, ver, v, lv;
        unsigned kn;
        double t;
        if (std::sscanf(line, "%d %d %d %u %255s %d %d %d %lf", &a, &b, &c, &kn, g, &ver, &v, &lv, &t) != 9) continue;
        if (a == im && b == jm && c == km && kn == knobs && gpu == g && ver == TUNE_VERSION) {
            *variant = v;
            *levels = lv;
            if (ms) *ms = t;
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

bool tune_put(const std::string& path, int im, int jm, int km, unsigned knobs, const std::string& gpu, int variant,
              int levels, double ms) {
    if (path.empty()) return false;
    // the parent directories, then keep every other key's lines and append this one (write + rename)
    for (size_t p = path.find('/', 1); p != std::string::npos; p = path.find('/', p + 1))
        mkdir(path.substr(0, p).c_str(), 0755);
    std::vector<std::string> keep;
    char line[512], g[256];
    if (FILE* f = std::fopen(path.c_str(), "r")) {
        while (std::fgets(line, sizeof(line), f)) {
            int a, b, c, ver, v, lv;
            unsigned kn;
            double t;
            if (std::sscanf(line, "%d %d %d %u %255s %d %d %d %lf", &a, &b, &c, &kn, g, &ver, &v, &lv, &t) != 9) continue;
            if (a == im && b == jm && c == km && kn == knobs && gpu == g) continue;
            keep.push_back(line);
        }
        std::fclose(f);
    }
    const std::string tmp = path + ".tmp." + std::to_string((long)getpid());
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) return false;
    for (const auto& l : keep) std::fputs(l.c_str(), f);
    std::fprintf(f, "%d %d %d %u %s %d %d %d %.6f\n", im, jm, km, knobs, gpu.c_str(), TUNE_VERSION, variant, levels, ms);
    const bool ok = std::fclose(f) == 0 && std::rename(tmp.c_str(), path.c_str()) == 0;
    if (!ok) std::remove(tmp.c_str());
    return ok;
}

unsigned tune_knobs(const atsat_dyn* h) {
    return (h->kc.turb ? 1u : 0u) | (h->kc.rad_on ? 2u : 0u) | (h->kc.precip_on ? 4u : 0u) | (h->kc.tmf_on ? 8u : 0u);
}

std::string device_name(const atsat_dyn* h) {
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) {
        cudaGetLastError();
        return tune_gpu_token(nullptr);
    }
    return tune_gpu_token(prop.name);
}

void tune_cache_store(atsat_dyn* h, double ms) {
    tune_put(tune_cache_path(nullptr), h->kc.im, h->kc.jm, h->kc.km, tune_knobs(h), device_name(h), h->variant,
             h->march_levels, ms);
}

// The march depth before any tuning: one run of all interior levels per (k, j) tile when the tiles alone
// give about two blocks per SM, else the levels split into runs so that they do.
// The compact rings of the march kernel's intermediate stages (three blocks per SM) apply where the stage
// streams at most 12 point arrays; ATSAT_MARCH_COMPACT=0 keeps the regular rings (two blocks per SM).
bool march_compact() {
    static const bool on = [] {
        const char* e = std::getenv("ATSAT_MARCH_COMPACT");
        return !(e && e[0] == '0' && e[1] == 0);
    }();
    return on;
}

// The default march depth: runs of radial levels such that the intermediate stage's blocks fill about 1.8
// waves of the resident blocks (measured best at 41x181x361, where the autotuner picks the same 13 levels).
int default_march_levels(const atsat_dyn* h) {
    const KConst& K = h->kc;
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess || nsm < 1) {
        cudaGetLastError();
        nsm = 152;
    }
    const int n_pt = 10 + (K.precip_on ? 1 : 0) + (K.rad_on ? 2 : 0) + (K.tmf_on ? 1 : 0);
    const int per_sm = (march_compact() && n_pt <= 12) ? 3 : 2;
    const int64_t tiles = (int64_t)((K.km - 1 + TILE_K - 1) / TILE_K) * ((K.jm - 4 + TILE_J - 1) / TILE_J);
    const int interior = K.im - 2;
    int64_t runs = tiles > 0 ? (int64_t)((double)per_sm * nsm * 1.8 / (double)tiles + 0.5) : 1;
    if (runs < 1) runs = 1;
    if (runs > interior) runs = interior;
    return (int)((interior + runs - 1) / runs);
}

// The radial march's stream per level: the stencil arrays' planes (y_n then the increment, w's low word
// after its y_n), and the point items nue, the nine frozen terms, the sources the knobs switch on and at the
// final stage dl_1, dl_2 of u, v, w, t.
MarchPlan make_plan_march(atsat_dyn* h, const MixedIO& io, int mode) {
    MarchPlan pl{};
    pl.err = h->dev_err;
    pl.wait_limit = h->wait_limit;
    pl.withhold = h->test_withhold;
    pl.levels = h->march_levels;
    pl.compact = march_compact();
    const bool dl = io.dl_in[0] != nullptr;
    int n = 0;
    auto halo = [&](const float* p) { pl.halo[n++] = arr_index(h, p); };
    halo(io.yn32[ATSAT_F_U]); if (dl) halo(io.dl_in[ATSAT_F_U]);
    halo(io.yn32[ATSAT_F_V]); if (dl) halo(io.dl_in[ATSAT_F_V]);
    halo(io.yn32[ATSAT_F_W]); halo(io.wlo); if (dl) halo(io.dl_in[ATSAT_F_W]);
    halo(io.yn32[ATSAT_F_T]); if (dl) halo(io.dl_in[ATSAT_F_T]);
    pl.n_halo = n;
    n = 0;
    auto pt = [&](const float* p) { if (n < MARCH_MAX_PT) pl.pt[n] = arr_index(h, p); return n++; };
    pt(io.nue);
    for (int f : {FZ_DPR, FZ_GU, FZ_BAN, FZ_BPS, FZ_DPTH, FZ_GV, FZ_DPPH, FZ_GW, FZ_DPS}) pt(io.fz[f]);
    pl.p_qprecip = h->kc.precip_on ? pt(io.q_precip) : -1;
    pl.p_rho = h->kc.rad_on ? pt(io.rho_mix) : -1;
    pl.p_qrad = h->kc.rad_on ? pt(io.q_rad) : -1;
    pl.p_tmf = h->kc.tmf_on ? pt(io.thermalmassflux) : -1;
    pl.p_dl = -1;
    if (mode == MODE_FINAL) {
        pl.p_dl = n;
        for (int q = 0; q < 4; q++) { pt(io.dl1[q]); pt(io.dl2[q]); }
    }
    pl.n_pt = n;
    return pl;
}

cudaError_t launch_stage(atsat_dyn* h, const MixedIO& io, const StageParams& sp, int mode) {
    const int v = (mode == MODE_RHS || !variant_available(h, h->variant)) ? ATSAT_DYN_STAGE_DIRECT : h->variant;
    switch (v) {
        case ATSAT_DYN_STAGE_TILED:
            return launch_rk_tile(h->maps, h->kf, io, sp, make_plan(h, io), mode, h->stream);
        case ATSAT_DYN_STAGE_SPLIT: return launch_rk_split(h->kf, io, sp, mode, 1, h->stream);
        case ATSAT_DYN_STAGE_SPLIT3: return launch_rk_split(h->kf, io, sp, mode, 3, h->stream);
        case ATSAT_DYN_STAGE_SPLIT13: return launch_rk_split(h->kf, io, sp, mode, 13, h->stream);
        case ATSAT_DYN_STAGE_SPLIT_TILED: {
            const cudaError_t e = launch_rk_mom(h->kf, io, sp, mode, h->stream);
            if (e != cudaSuccess) return e;
            const TracerPlan pl = make_plan_tracer(h, io, mode);
            if (pl.n_items != tracer_plan_items(mode, io.dl_in[0] != nullptr, h->kc.turb != 0))
                return cudaErrorInvalidValue;   // the plan and the kernel disagree: never expected
            return launch_rk_tracer_tile(h->maps, h->kf, io, sp, pl, mode, h->stream);
        }
        case ATSAT_DYN_STAGE_TILED2: {
            const TracerPlan pm = make_plan_mom(h, io);
            const TracerPlan pt = make_plan_tracer(h, io, mode);
            const bool dl = io.dl_in[0] != nullptr;
            if (pm.n_items != mom_plan_items(dl) || pt.n_items != tracer_plan_items(mode, dl, h->kc.turb != 0))
                return cudaErrorInvalidValue;   // the plans and the kernels disagree: never expected
            const cudaError_t e = launch_rk_mom_tile(h->maps, h->kf, io, sp, pm, mode, h->stream);
            if (e != cudaSuccess) return e;
            return launch_rk_tracer_tile(h->maps, h->kf, io, sp, pt, mode, h->stream);
        }
        case ATSAT_DYN_STAGE_MARCH: {
            const MarchPlan pm = make_plan_march(h, io, mode);
            const TracerPlan pt = make_plan_tracer(h, io, mode);
            if (pt.n_items != tracer_plan_items(mode, io.dl_in[0] != nullptr, h->kc.turb != 0))
                return cudaErrorInvalidValue;   // the plan and the kernel disagree: never expected
            const cudaError_t e = launch_rk_mom_march(h->maps, h->kf, io, sp, pm, mode, h->stream);
            if (e != cudaSuccess) return e;
            return launch_rk_tracer_tile(h->maps, h->kf, io, sp, pt, mode, h->stream);
        }
        default: return launch_rk_stage_mixed(h->kf, io, sp, mode, h->stream);
    }
}

// resident: called from atsat_dyn_iterate, which keeps the FP32 copies of the next y_n up to date and
// ends each iteration with the live and n-level fields equal.
int enqueue_rk4_mixed(atsat_dyn* h, bool resident) {
    int rc;
    if ((rc = do_level_metric(h))) return rc;
    double* yn[NPROG];
    double* L[NPROG];
    for (int q = 0; q < NPROG; q++) { yn[q] = h->f[ATSAT_F_N_BASE + q]; L[q] = h->f[q]; }
    const bool fast = resident && h->aliased && h->shadow_valid;
    // fields whose live values differ from y_n although the run is aliased (split after restoreVar)
    const uint32_t split = fast ? h->split_mask : 0u;
    const uint32_t all = (1u << NPROG) - 1u;
    if (fast && (h->edges_dirty & ~split)) {
        // live == y_n: the cells no stage writes must hold a zero increment in A, B and C (contiguous)
        CK(h, cudaMemsetAsync(h->dlA[0], 0, (size_t)3 * NPROG * h->kc.fsz * sizeof(float), h->stream));
        h->edges_dirty = 0;
    }
    if (split) {
        // stage 0 reads C: zero for the aliased fields, live - y_n for the split ones (the prepare's dl_0,
        // which also writes their A and B at the cells no stage writes)
        CK(h, cudaMemsetAsync(h->dlC[0], 0, (size_t)NPROG * h->kc.fsz * sizeof(float), h->stream));
    }
    if ((rc = enqueue_mixed_prepare(h, yn, fast ? split : all, fast))) return rc;
    if (resident && (!fast || split)) {
        // the copies of y_{n+1} start as (float) live: cells the step and the BCs leave alone keep them
        // (every field on the general path, the split ones on the aliased path)
        MixedPrep pr{};
        pr.write_yn32 = 1;
        for (int q = 0; q < NPROG; q++) {
            pr.yn64[q] = L[q];
            pr.live64[q] = L[q];
            pr.yn32[q] = (!fast || ((split >> q) & 1u)) ? h->yo32[q] : nullptr;
        }
        pr.wlo = pr.yn32[ATSAT_F_W] ? h->wlo_o : nullptr;
        pr.skip_frozen = 1;
        Timed t(h, ATSAT_K_PREPARE);
        CK(h, launch_mixed_prepare(h->kc, pr, h->stream));
        h->launches += 1;
    }
    const double dt = h->p.dt;
    // increments: stage 0 reads dl_0 (C; none when live == y_n) and writes dl_1 to A, stage 1: A -> B,
    // stage 2: B -> C, the final stage reads C and the point values of A and B
    float* const* ins[4] = {(fast && !split) ? nullptr : h->dlC, h->dlA, h->dlB, h->dlC};
    float* const* outs[4] = {h->dlA, h->dlB, h->dlC, nullptr};
    for (int stage = 0; stage < 4; stage++) {
        StageParams sp{};
        sp.stage = stage;
        sp.write_all_rhs = h->write_all_rhs;
        sp.c_in = (stage == 0 || stage == 1) ? 0.5 * dt : (stage == 2 ? dt : 0.0);
        sp.wgt = (stage == 0 || stage == 3) ? 1.0 : 2.0;
        sp.sixth_dt = dt / 6.0;
        sp.c_in_f = (float)sp.c_in;
        sp.wgt_f = (float)sp.wgt;
        sp.sixth_dt_f = (float)sp.sixth_dt;
        MixedIO io = make_mixed_io(h, ins[stage], outs[stage], stage == 3 ? L : nullptr);
        if (stage == 3 && resident) {
            for (int q = 0; q < NPROG; q++) io.out32[q] = h->yo32[q];
            io.wlo_out = h->wlo_o;
        }
        Timed t(h, ATSAT_K_RK_STAGE);
        CK(h, launch_stage(h, io, sp, stage == 3 ? MODE_FINAL : MODE_STAGE));
        h->launches += launches_per_stage(h);
        // the TMA-tiled tracer kernel leaves the final stage's FP64 sum to launch_final_combine
        const int v = variant_available(h, h->variant) ? h->variant : ATSAT_DYN_STAGE_DIRECT;
        if (stage == 3 && (v == ATSAT_DYN_STAGE_SPLIT_TILED || v == ATSAT_DYN_STAGE_TILED2 || v == ATSAT_DYN_STAGE_MARCH))
            h->launches += 1;
    }
    return ATSAT_DYN_OK;
}

int enqueue_pressure(atsat_dyn* h, int sweeps) {
    const KConst& K = h->kc;
    {
        Timed t(h, ATSAT_K_PRESS_BOUNDARY);
        CK(h, launch_projection_prep(K, h->six, h->stream));
        h->launches += 2;
    }
    CK(h, cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), h->stream));
    const bool incr = K.press_incr;
    {
        Timed t(h, ATSAT_K_PRESS_SOURCE);
        CK(h, launch_press_source(K, h->geo, incr ? h->f[ATSAT_F_RHS_U] : h->f[ATSAT_F_AUX_U],
                                  incr ? h->f[ATSAT_F_RHS_V] : h->f[ATSAT_F_AUX_V],
                                  incr ? h->f[ATSAT_F_RHS_W] : h->f[ATSAT_F_AUX_W], h->f[ATSAT_F_AUX_U],
                                  h->f[ATSAT_F_AUX_V], h->f[ATSAT_F_AUX_W], h->f[ATSAT_F_RHS_U], h->f[ATSAT_F_RHS_V],
                                  h->f[ATSAT_F_RHS_W], h->f[ATSAT_F_P_DYN], h->src, h->counter, h->stream));
        h->launches += 1;
    }
    const bool line = h->p.press_line != 0, baro = h->p.press_baro != 0;
    double* pd = h->f[ATSAT_F_P_DYN];
    if (line) {                 // the interior mean on entry, held after every sweep
        Timed t(h, ATSAT_K_PRESS_BOUNDARY);
        int n = 0;
        CK(h, launch_interior_mean(K, pd, h->imean_partial, h->pmean, h->stream, &n));
        h->launches += n;
    }
    for (int s = 0; s < sweeps; s++) {
        for (int colour = 0; colour < 2; colour++) {
            Timed t(h, ATSAT_K_PRESS_SWEEP);
            CK(h, launch_press_sweep(K, h->geo, h->src, pd, colour, h->stream));
            h->launches += ((K.km - 1) & 1) ? 2 : 1;     // odd km-1: the seam cells follow their partner
        }
        if (line) {
            for (int colour = 0; colour < 2; colour++) {
                Timed t(h, ATSAT_K_PRESS_SWEEP);
                int n = 0;
                CK(h, launch_line_pass(K, h->geo, h->src, pd, h->line_cp, h->line_dp, colour, h->stream, &n));
                h->launches += n;
            }
        }
        if (baro) {
            Timed t(h, ATSAT_K_PRESS_SWEEP);
            int n = 0;
            CK(h, launch_barotropic(K, h->geo, h->src, pd, h->baro, h->stream, &n));
            h->launches += n;
        }
        Timed t(h, ATSAT_K_PRESS_BOUNDARY);
        CK(h, launch_press_boundary(K, pd, h->stream));
        h->launches += 1;
        if (line) {
            int n = 0;
            CK(h, launch_interior_mean(K, pd, h->imean_partial, h->pmean + 1, h->stream, &n));
            CK(h, launch_mean_shift(K, pd, h->pmean, h->stream));
            h->launches += n + 1;
        }
    }
    return ATSAT_DYN_OK;
}

// restoreVar. In a resident mixed run the n-level fields become aliases of the live ones (no copy)
// and the FP32 copy of y_{n+1} becomes the next step's copy of y_n.
int enqueue_restore(atsat_dyn* h, bool resident = false) {
    Timed t(h, ATSAT_K_GLUE);
    const size_t bytes = (size_t)h->kc.fsz * 8;
    if (resident && h->p.precision == ATSAT_DYN_MIXED) {
        if (h->aliased) {
            // the split fields share their live storage again (spare_n keeps their buffers)
            for (int q = 0; q < NPROG; q++)
                if ((h->split_mask >> q) & 1u) h->f[ATSAT_F_N_BASE + q] = h->f[q];
            h->split_mask = 0;
        } else {
            for (int q = 0; q < NPROG; q++) {
                h->spare_n[q] = h->f[ATSAT_F_N_BASE + q];
                h->f[ATSAT_F_N_BASE + q] = h->f[q];
            }
            h->aliased = true;
            h->split_mask = 0;
            // both FP32 copies must agree on the cells no step or boundary pass writes
            const size_t b32 = (size_t)h->kc.fsz * 4;
            for (int q = 0; q < NPROG; q++)
                CK(h, cudaMemcpyAsync(h->yn32[q], h->yo32[q], b32, cudaMemcpyDeviceToDevice, h->stream));
            CK(h, cudaMemcpyAsync(h->wlo, h->wlo_o, b32, cudaMemcpyDeviceToDevice, h->stream));
        }
        for (int q = 0; q < NPROG; q++) std::swap(h->yn32[q], h->yo32[q]);
        std::swap(h->wlo, h->wlo_o);
        h->shadow_valid = true;
    } else {
        for (int q = 0; q < NPROG; q++)
            CK(h, cudaMemcpyAsync(h->f[ATSAT_F_N_BASE + q], h->f[q], bytes, cudaMemcpyDeviceToDevice, h->stream));
    }
    CK(h, cudaMemcpyAsync(h->f[ATSAT_F_P_DYNN], h->f[ATSAT_F_P_DYN], bytes, cudaMemcpyDeviceToDevice, h->stream));
    return ATSAT_DYN_OK;
}

// Give the n-level fields their own buffers again (a copy of the shared values) before any call that
// can observe the live and n-level fields separately. `overwritten[q]`: n-level field q is about to be
// replaced as a whole (an upload), so its buffer needs no copy.
int unalias(atsat_dyn* h, const bool* overwritten = nullptr) {
    if (!h->aliased) return ATSAT_DYN_OK;
    const size_t bytes = (size_t)h->kc.fsz * 8;
    for (int q = 0; q < NPROG; q++) {
        if ((h->split_mask >> q) & 1u) continue;           // has its own n-level storage already
        if (!(overwritten && overwritten[q]))
            CK(h, cudaMemcpyAsync(h->spare_n[q], h->f[q], bytes, cudaMemcpyDeviceToDevice, h->stream));
        h->f[ATSAT_F_N_BASE + q] = h->spare_n[q];
    }
    h->aliased = false;
    h->shadow_valid = false;
    h->split_mask = 0;
    return ATSAT_DYN_OK;
}

// In an aliased resident run, give the fields of `mask` their own n-level storage again (a copy of the
// shared values), the others staying aliased: for a call after restoreVar that changes those live fields
// alone. The FP32 copies of y_n stay valid.
int split_fields(atsat_dyn* h, uint32_t mask) {
    if (!h->aliased) return ATSAT_DYN_OK;
    const size_t bytes = (size_t)h->kc.fsz * 8;
    for (int q = 0; q < NPROG; q++) {
        if (!((mask >> q) & 1u) || ((h->split_mask >> q) & 1u)) continue;
        CK(h, cudaMemcpyAsync(h->spare_n[q], h->f[q], bytes, cudaMemcpyDeviceToDevice, h->stream));
        h->f[ATSAT_F_N_BASE + q] = h->spare_n[q];
    }
    h->split_mask |= mask;
    return ATSAT_DYN_OK;
}

int enqueue_bc(atsat_dyn* h, bool resident = false) {
    Timed t(h, ATSAT_K_GLUE);
    float* s32[ATSAT_NFIELDS] = {};
    const bool mixed = h->p.precision == ATSAT_DYN_MIXED;
    const bool shadows = resident && mixed;
    if (shadows)
        for (int q = 0; q < NPROG; q++) s32[q] = h->yo32[q];
    // the FP32 copies of the point inputs the boundary passes write are refreshed in the same threads
    // when they are current; otherwise they are rebuilt before the next step
    const int bc_inputs[6] = {ATSAT_F_NUE, ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH,
                              ATSAT_F_FLUXLIM_NH4SH, ATSAT_F_THERMALMASSFLUX};
    if (mixed)
        for (int fid : bc_inputs) {
            const int slot = conv_slot(fid);
            if (slot >= 0 && !h->conv_dirty[slot]) s32[fid] = h->conv32[slot];
        }
    CK(h, launch_boundary_conditions(h->kc, h->p, h->f, mixed ? s32 : nullptr, shadows ? h->wlo_o : nullptr,
                                     h->stream));
    h->launches += 3;
    return ATSAT_DYN_OK;
}

// AtomUtils::damp_wiggles (lib/Utils.cpp:229-322) on a device field, the pressure source as the copy
int enqueue_damp(atsat_dyn* h, int fid, bool ai, bool aj, bool ak, double strength, int passes) {
    Timed t(h, ATSAT_K_GLUE);
    const KConst& K = h->kc;
    const size_t bytes = (size_t)K.fsz * 8;
    const double coeff = strength * 0.25;
    const int seam = (h->p.phi_periodic && K.km > 2) ? 1 : 0;
    double* f = h->f[fid];
    for (int pass = 0; pass < passes; pass++) {
        const bool axes[3] = {ak, aj, ai};
        for (int a = 0; a < 3; a++) {
            if (!axes[a]) continue;
            CK(h, cudaMemcpyAsync(h->src, f, bytes, cudaMemcpyDeviceToDevice, h->stream));
            CK(h, launch_damp_axis(K, h->src, f, coeff, a, seam, h->stream));
            h->launches += 1;
        }
    }
    mark_dirty(h, fid);
    return ATSAT_DYN_OK;
}

// the p_dyn filter of cSaturnModel::Run after the pressure call (cSaturnModel.cpp:894-897)
int enqueue_damp_pdyn(atsat_dyn* h) {
    switch (h->p.damp_pdyn) {
        case 1: return enqueue_damp(h, ATSAT_F_P_DYN, true, true, true, 1.0, 1);
        case 2: return enqueue_damp(h, ATSAT_F_P_DYN, true, false, false, 1.0, 1);
        case 3: return enqueue_damp(h, ATSAT_F_P_DYN, true, false, true, 1.0, 1);
        default: return ATSAT_DYN_OK;
    }
}

const int CLAMP_SPECIES[11] = {ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                               ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                               ATSAT_F_CH4_ICE, ATSAT_F_NH4SH};

// cSaturnModel::clampNegativeSpecies (FileIO_Sat.cpp:716-772); resident mixed runs also floor the FP32
// copies of y_{n+1} that the next step starts from
int enqueue_clamp(atsat_dyn* h, bool resident = false) {
    if (!h->p.clamp_species) return ATSAT_DYN_OK;
    Timed t(h, ATSAT_K_GLUE);
    double* f[11];
    float* s32[11];
    const bool shadows = resident && h->p.precision == ATSAT_DYN_MIXED;
    for (int q = 0; q < 11; q++) {
        f[q] = h->f[CLAMP_SPECIES[q]];
        s32[q] = shadows ? h->yo32[CLAMP_SPECIES[q]] : nullptr;
    }
    CK(h, launch_clamp_species(h->kc, f, shadows ? s32 : nullptr, h->clamp_added, h->clamp_cells, h->clamp_partial,
                               h->stream));
    h->launches += 2;
    return ATSAT_DYN_OK;
}

}  // namespace

extern "C" {

int atsat_dyn_abi_version(void) { return ATSAT_DYN_ABI_VERSION; }

int atsat_dyn_params_default(atsat_dyn_params* p) {
    if (!p) return ATSAT_DYN_E_INVALID;
    memset(p, 0, sizeof(*p));
    // the committed configuration (cli/config_atsat.xml) and cSaturnModel.h member initialisers
    p->re = 100000.0; p->pr = 69.0;
    p->sc_h2o = 0.61; p->sc_nh3 = 0.61; p->sc_h2s = 0.94; p->sc_ch4 = 0.99; p->sc_nh4sh = 0.7;
    p->u_0 = 470.0; p->t_ref = 134.0; p->L_atm = 500.0; p->g = 10.0; p->omega = 0.000163;
    p->Coriolis = 1.0; p->centrifugal = 1.0; p->buoyancy = 1.0; p->chemical_reaction = 1.0;
    // ChemistrySat::ThermalPropertiesSat of the default composition (ChemistrySat.h:475-530)
    p->cp_mix = 0x1.3a544e8a8f013p+13;
    p->r_mix = 1.382;
    p->R_mix = 0x1.6ba7dd06e410fp+11;
    p->dt = 0.01;
    p->metric_radius_km = 58232.0; p->sinthe_min = 0.0; p->buoy_scale = 1.0; p->turb_coupling = 1.0;
    p->rad_coupling = 0.0; p->precip_coupling = 1.0; p->thermal_massflux = 0.0; p->species_divu = 0.0;
    p->pdyn_cap = 0.2;
    p->phi_periodic = 1; p->metric_split = 1; p->coriolis_split = 1; p->hydro_buoy = 0;
    p->nd_cor = 1; p->nd_cent = 0; p->nd_buoy = 0; p->cell_hold = 1; p->adiabatic = 1; p->adiabatic_rho = 1;
    p->turb_active = 1; p->t_limiter = 0; p->buoy_legacy = 0; p->chrom = 0; p->cp_h2_dyn = 0; p->print_diag = 0;
    p->coord_stretching = 0;
    p->press_src = 1; p->press_incr = 1; p->press_sweeps = 1; p->press_wall = 0; p->rigid_lid = 1;
    p->press_line = 0; p->press_baro = 0; p->precision = ATSAT_DYN_FP64;
    p->bc_radius_form = 2; p->bc_bottom_form = 3; p->bc_pole_form = 1; p->bc_pole_fill = 1; p->bc_lid_u = 1;
    p->bc_top_taper = 2; p->bc_species_lid_copy = 1; p->bc_species_wall_copy = 2; p->local_rho = 1;
    p->damp_pdyn = 3; p->clamp_species = 1; p->driver_glue = 0; p->press_every_step = 0;
    return ATSAT_DYN_OK;
}

static const char* envs(const char* n) { return getenv(n); }
static int env_i(const char* n, int d) { const char* e = envs(n); return e ? atoi(e) : d; }
static double env_d(const char* n, double d) { const char* e = envs(n); return e ? atof(e) : d; }

int atsat_dyn_params_from_env(atsat_dyn_params* p) {
    if (!p) return ATSAT_DYN_E_INVALID;
    // the knobs as the reference resolves them; see the file:line of each field in atsat_dyn.h
    p->metric_radius_km = env_d("ATSAT_METRIC_RADIUS", 58232.0);
    { const double x = env_d("ATSAT_SINTHE_MIN", 0.0); p->sinthe_min = (x >= 0.0 && x < 1.0) ? x : 0.0; }
    p->buoy_scale = env_d("ATSAT_BUOY_SCALE", 1.0);
    p->turb_coupling = env_d("ATSAT_TURB_COUPLING", 1.0);
    p->rad_coupling = env_d("ATSAT_RAD_COUPLING", 0.0);
    p->precip_coupling = env_d("ATSAT_PRECIP_COUPLING", 1.0);
    p->thermal_massflux = env_d("ATSAT_THERMAL_MASSFLUX", 0.0);
    p->species_divu = env_d("ATSAT_SPECIES_DIVU", 0.0);
    p->pdyn_cap = env_d("ATSAT_PDYN_CAP", 0.2);
    p->phi_periodic = env_i("ATSAT_BC_PHI_PERIODIC", 1) != 0;
    p->metric_split = envs("ATSAT_METRIC_SPLIT") ? (env_i("ATSAT_METRIC_SPLIT", 1) != 0) : 1;
    p->coriolis_split = (envs("ATSAT_CORIOLIS_SPLIT") ? (env_i("ATSAT_CORIOLIS_SPLIT", 1) != 0) : 1) && p->metric_split;
    const int geo = envs("ATSAT_GEO_BALANCE") ? (env_i("ATSAT_GEO_BALANCE", 1) != 0) : 1;
    p->hydro_buoy = (envs("ATSAT_HYDRO_BUOY") ? (env_i("ATSAT_HYDRO_BUOY", 0) != 0) : 0) && p->metric_split;
    const int nd_all = env_i("ATSAT_NONDIM", 0);
    const int c_cor = envs("ATSAT_ND_COR") ? env_i("ATSAT_ND_COR", 0) : (geo ? 1 : -1);
    const int c_cent = env_i("ATSAT_ND_CENT", -1);
    const int c_buoy = env_i("ATSAT_ND_BUOY", -1);
    p->nd_cor = ((c_cor >= 0 ? c_cor : nd_all) != 0);
    p->nd_cent = ((c_cent >= 0 ? c_cent : nd_all) != 0);
    p->nd_buoy = ((c_buoy >= 0 ? c_buoy : nd_all) != 0);
    p->cell_hold = envs("ATSAT_CELL_HOLD") ? (env_i("ATSAT_CELL_HOLD", 0) != 0) : geo;
    p->adiabatic = envs("ATSAT_ADIABATIC") ? (env_i("ATSAT_ADIABATIC", 1) != 0) : 1;
    p->adiabatic_rho = envs("ATSAT_ADIABATIC_RHO") ? (env_i("ATSAT_ADIABATIC_RHO", 1) != 0) : 1;
    {
        const int turb_env = env_i("ATSAT_TURB", -1);
        const char* tm = envs("ATSAT_TURB_MODEL");
        const std::string model = tm ? tm : "k_omega_SST";
        p->turb_active = (turb_env != 0) && !(model.empty() || model == "none" || model == "laminar");
    }
    p->t_limiter = env_i("ATSAT_T_LIMITER", 0) != 0;
    p->buoy_legacy = env_i("ATSAT_BUOY_LEGACY", 0) != 0;
    p->chrom = envs("ATSAT_CHROM") && env_i("ATSAT_CHROM", 0) != 0;
    p->cp_h2_dyn = (env_i("ATSAT_CP_H2", 0) != 0) || (env_i("ATSAT_CP_GAS", 0) != 0);
    p->print_diag = env_i("ATSAT_TB_DIAG", 0) > 0 || env_i("ATSAT_UB_DIAG", 0) > 0 || env_i("ATSAT_CWB_DIAG", 0) > 0;
    p->press_src = env_i("ATSAT_PRESS_SRC", 1);
    // Run() sets ATSAT_PRESS_INCR=1 under GEO_BALANCE unless it is given (cSaturnModel.cpp:612)
    p->press_incr = envs("ATSAT_PRESS_INCR") ? (env_i("ATSAT_PRESS_INCR", 0) != 0) : geo;
    { const int n = env_i("ATSAT_PRESS_SWEEPS", 1); p->press_sweeps = n > 0 ? n : 1; }
    p->press_wall = env_i("ATSAT_PRESS_WALL", 0) != 0;
    p->rigid_lid = env_i("ATSAT_BC_RIGID_LID", 1) != 0;
    p->press_line = env_i("ATSAT_PRESS_LINE", 0) != 0;
    {   // under HYDRO_BUOY Run() sets ATSAT_PRESS_BAROTROPIC=1 unless given (cSaturnModel.cpp:615)
        const int raw = envs("ATSAT_PRESS_BAROTROPIC") ? env_i("ATSAT_PRESS_BAROTROPIC", 0) : (p->hydro_buoy ? 1 : 0);
        p->press_baro = (raw != 0) && p->phi_periodic && !p->press_wall;
    }
    p->bc_radius_form = env_i("ATSAT_BC_RADIUS_COPY", 2);
    p->bc_bottom_form = env_i("ATSAT_BC_BOTTOM_FORM", 3);
    p->bc_pole_form = env_i("ATSAT_BC_POLE_COPY", 1);
    p->bc_pole_fill = env_i("ATSAT_BC_POLE_FILL", 1);
    p->bc_lid_u = env_i("ATSAT_BC_LID_U", p->rigid_lid);
    p->bc_top_taper = env_i("ATSAT_BC_TOP_TAPER", 2);
    p->bc_species_lid_copy = env_i("ATSAT_BC_SPECIES_LID_COPY", 1);
    p->bc_species_wall_copy = env_i("ATSAT_BC_SPECIES_WALL_COPY", 2);
    p->local_rho = envs("ATSAT_LOCAL_RHO") ? (env_i("ATSAT_LOCAL_RHO", 1) != 0) : 1;
    // the driver's glue (cSaturnModel.cpp:894; FileIO_Sat.cpp:717)
    p->damp_pdyn = envs("ATSAT_DAMP_PDYN") ? env_i("ATSAT_DAMP_PDYN", 0) : (geo ? 3 : 1);
    p->clamp_species = env_i("ATSAT_NO_CLAMP", 0) ? 0 : 1;
    if (env_i("ATSAT_BC_SEAM_DAMP", 0) != 0 || env_i("ATSAT_BC_T_LID_PIN", 0) != 0) return ATSAT_DYN_E_UNSUPPORTED;
    return ATSAT_DYN_OK;
}

// Device tables of the pressure variants, built with the reference's own expressions
// (PressureSolver.h:150-162, 310-316, 578-580, 613-616, 640-644).
int setup_press_variants(atsat_dyn* h) {
    const KConst& K = h->kc;
    const atsat_dyn_params& p = h->p;
    const bool line = p.press_line != 0, baro = p.press_baro != 0;
    if (!line && !baro) return ATSAT_DYN_OK;
    constexpr double PI = 3.14159265358979323846;
    const int N = K.km - 1, J = K.jm - 2, NM = N / 2;
    const int64_t n_line = line ? 2 * K.fsz : 0;
    const int64_t n_mean = line ? interior_mean_partials(K) + 2 : 0;
    const int64_t n_tab = baro ? 2LL * (NM + 1) * N + (NM + 1) + K.jm + J : 0;
    const int64_t n_scr = baro ? (int64_t)J * N + J + 4LL * (NM + 1) * J : 0;
    const int64_t total = n_line + n_mean + n_tab + n_scr + 64;
    cudaError_t e = cudaMalloc(&h->pv_buf, (size_t)total * 8);
    if (e != cudaSuccess) { h->pv_buf = nullptr; return fail(h, ATSAT_DYN_E_NOMEM, "pressure variants: %s", cudaGetErrorString(e)); }
    double* q = h->pv_buf;
    if (line) {
        h->line_cp = q; q += K.fsz;
        h->line_dp = q; q += K.fsz;
        h->pmean = q; q += 2;
        h->imean_partial = q; q += interior_mean_partials(K);
    }
    if (baro) {
        std::vector<double> tab((size_t)n_tab);
        double* ct = tab.data();
        double* st = ct + (size_t)(NM + 1) * N;
        double* lam = st + (size_t)(NM + 1) * N;
        double* sinthe = lam + (NM + 1);
        double* abs_sin = sinthe + K.jm;
        for (int mm = 0; mm <= NM; mm++) {
            for (int k = 0; k < N; k++) {
                const double a = 2.0 * PI * (double)((long)mm * k % N) / N;
                ct[(size_t)mm * N + k] = std::cos(a);
                st[(size_t)mm * N + k] = std::sin(a);
            }
            const double sl = std::sin(PI * mm / N);
            lam[mm] = 4.0 * sl * sl * K.inv_dphi2;
        }
        for (int j = 0; j < K.jm; j++) {
            double sv = std::sin(h->the_z[j]);
            if (sv < p.sinthe_min) sv = p.sinthe_min;
            if (sv == 0.0) sv = 1.0e-5;
            sinthe[j] = sv;
        }
        for (int jj = 0; jj < J; jj++) abs_sin[jj] = std::fabs(std::sin(h->the_z[jj + 1]));
        double A2 = 0.0;
        for (int i = 1; i < K.im - 1; i++) {
            const double rm = metric_radius(p, h->rad_z[i]);
            A2 += 1.0 / (rm * rm);
        }
        double* dtab = q; q += n_tab;
        e = cudaMemcpy(dtab, tab.data(), (size_t)n_tab * 8, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(h, ATSAT_DYN_E_CUDA, "pressure variant tables: %s", cudaGetErrorString(e));
        BaroTables& T = h->baro;
        T.A2 = A2;
        T.ct = dtab;
        T.st = dtab + (size_t)(NM + 1) * N;
        T.lam = T.st + (size_t)(NM + 1) * N;
        T.sinthe = T.lam + (NM + 1);
        T.abs_sin = T.sinthe + K.jm;
        T.R = q; q += (int64_t)J * N;
        T.ra = q; q += J;
        T.Ac = q; q += (int64_t)(NM + 1) * J;
        T.As = q; q += (int64_t)(NM + 1) * J;
        T.cp = q; q += (int64_t)(NM + 1) * J;
        T.dp = q; q += (int64_t)(NM + 1) * J;
    }
    return ATSAT_DYN_OK;
}

// The closure's buffers and tables (Turbulence.h:243-269 geometry, cSaturnModel.h:1062-1074, 686-692).
int setup_turbulence(atsat_dyn* h) {
    const KConst& K = h->kc;
    const atsat_dyn_params& p = h->p;
    const atsat_dyn_grid& g = h->g;
    const int im = K.im, jm = K.jm;
    const int64_t n_tab = 5LL * im + 2LL * jm + (int64_t)im * jm;
    const int64_t total = K.fsz + (int64_t)jm * K.kp + n_tab + 16;
    cudaError_t e = cudaMalloc(&h->turb_buf, (size_t)total * 8);
    if (e != cudaSuccess) { h->turb_buf = nullptr; return fail(h, ATSAT_DYN_E_NOMEM, "turbulence: %s", cudaGetErrorString(e)); }
    e = cudaMemset(h->turb_buf, 0, (size_t)total * 8);
    if (e != cudaSuccess) return fail(h, ATSAT_DYN_E_CUDA, "turbulence: %s", cudaGetErrorString(e));
    double* q = h->turb_buf;
    h->turb_prod = q; q += K.fsz;
    h->turb_vs = q; q += (int64_t)jm * K.kp;
    std::vector<double> t((size_t)n_tab);
    double* rm = t.data();
    double* inv_rm = rm + im;
    double* inv_rm2dthe = inv_rm + im;
    double* height = inv_rm2dthe + im;
    double* thick = height + im;
    double* sinthe = thick + im;
    double* cot = sinthe + jm;
    double* irs = cot + jm;
    const float hl = (float)(p.L_atm * g.dr);           // the model's float layer spacing, km
    const double inv_2dthe = 1.0 / (2.0 * g.dthe), inv_2dphi = 1.0 / (2.0 * g.dphi);
    for (int i = 0; i < im; i++) {
        rm[i] = metric_radius(p, h->rad_z[i]);
        inv_rm[i] = 1.0 / rm[i];
        inv_rm2dthe[i] = inv_2dthe / rm[i];
        height[i] = (double)((float)i * hl) * 1.0e3;
        thick[i] = (i > im - 2) ? 0.0 : (double)((float)(i + 1) * hl - (float)i * hl) * 1.0e3;
    }
    for (int j = 0; j < jm; j++) {
        double sv = std::sin(h->the_z[j]);
        if (sv == 0.0) sv = 1.0e-5;
        sinthe[j] = sv;
        cot[j] = std::cos(h->the_z[j]) / sv;
    }
    for (int i = 0; i < im; i++)
        for (int j = 0; j < jm; j++) irs[(size_t)i * jm + j] = inv_2dphi / (rm[i] * sinthe[j]);
    double* d = q;
    e = cudaMemcpy(d, t.data(), (size_t)n_tab * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(h, ATSAT_DYN_E_CUDA, "turbulence tables: %s", cudaGetErrorString(e));
    TurbTables& T = h->ttab;
    T.rm = d; T.inv_rm = d + im; T.inv_rm2dthe = d + 2 * im; T.height_m = d + 3 * im; T.thick_m = d + 4 * im;
    T.sinthe = d + 5 * im; T.cotanthe = d + 5 * im + jm; T.inv_rmsinthe2dphi = d + 5 * im + 2 * jm;
    T.dr = g.dr; T.dthe = g.dthe; T.dphi = g.dphi;
    return ATSAT_DYN_OK;
}

// the ABL taper's layer step (Turbulence.h:569-574), from the model's float layer table
double turb_taper_dz(const atsat_dyn* h) {
    const int im = h->kc.im;
    const float hl = (float)(h->p.L_atm * h->g.dr);
    auto height = [&](int i) { return (double)((float)i * hl) * 1.0e3; };
    int i_abl = 0;
    while (i_abl < im - 1 && height(i_abl) <= h->tp.abl_height) i_abl++;
    const double a = height(i_abl < im - 1 ? i_abl : im - 1), b = height(i_abl - 1 > 0 ? i_abl - 1 : 0);
    return std::max(1.0, a - b);
}

// Turbulence<cSaturnModel>::run on the device fields. It runs after restoreVar and changes the live k* and
// omega* only, so the next step starts from the n-level values restoreVar saved (its y_n) with the live
// ones as its stage-0 input (RungeKutta_Sat_Turb.cpp:250-320). A resident mixed run shares the live and
// n-level storage after restoreVar, so it gives the n-level fields their own copies first; the next step
// then rebuilds its FP32 copies of y_n and the stage-0 increment live - y_n.
int enqueue_turbulence(atsat_dyn* h, bool resident = false) {
    if (!h->turb_buf) {
        int rc = setup_turbulence(h);
        if (rc) return rc;
    }
    if (resident && h->p.precision == ATSAT_DYN_MIXED) {
        // the closure changes live k* and omega* only (and their n-level copies at the seam and corners):
        // those two get their own n-level storage, the other fields stay aliased
        int rc = split_fields(h, (1u << ATSAT_F_TKE) | (1u << ATSAT_F_DIS));
        if (rc) return rc;
    }
    h->ttab.taper_dz = turb_taper_dz(h);
    {
        Timed t(h, ATSAT_K_GLUE);
        int n = 0;
        CK(h, launch_turbulence(h->kc, h->p, h->tp, h->ttab, h->f, h->turb_prod, h->turb_vs, h->stream, &n));
        h->launches += n;
    }
    for (int fid : {ATSAT_F_NUE, ATSAT_F_TKE_SOURCE, ATSAT_F_DIS_SOURCE}) mark_dirty(h, fid);
    return ATSAT_DYN_OK;
}

int atsat_dyn_create(const atsat_dyn_grid* g, const atsat_dyn_params* p, atsat_dyn_t* out) {
    if (!g || !p || !out || !g->rad_z || !g->the_z) return ATSAT_DYN_E_INVALID;
    *out = nullptr;
    if (g->im < 5 || g->jm < 7 || g->km < 5 || g->im > 4096 || g->jm > 65536 || g->km > 65536)
        return ATSAT_DYN_E_INVALID;
    atsat_dyn* h = new atsat_dyn();
    h->g = *g;
    h->rad_z.assign(g->rad_z, g->rad_z + g->im);
    h->the_z.assign(g->the_z, g->the_z + g->jm);
    h->g.rad_z = h->rad_z.data();
    h->g.the_z = h->the_z.data();
    h->p = *p;
    int rc = check_supported(h, *p);
    if (rc) { *out = h; return rc; }
    build_constants(h);
    build_geometry(h, nullptr, nullptr);
    build_mixed_constants(h);
    const KConst& K = h->kc;
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        fail(h, e == cudaErrorMemoryAllocation ? ATSAT_DYN_E_NOMEM : ATSAT_DYN_E_CUDA, "%s: %s", what,
             cudaGetErrorString(e));
        *out = h;
        return e == cudaErrorMemoryAllocation ? ATSAT_DYN_E_NOMEM : ATSAT_DYN_E_CUDA;
    };
    cudaError_t e;
    if ((e = cudaGetDevice(&h->device)) != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamCreate");
    {
        // host memory the SMs may address in place: both attributes, not just HMM's page migration
        int pageable = 0, host_tables = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->device) != cudaSuccess ||
            cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device) !=
                cudaSuccess) {
            cudaGetLastError();
            pageable = host_tables = 0;
        }
        h->host_ok = pageable == 1 && host_tables == 1;
        const char* env = std::getenv("ATSAT_HOST_DIRECT");
        h->host_direct = h->host_ok && !(env && std::strcmp(env, "0") == 0);
        const char* as = std::getenv("ATSAT_DYN_ASYNC");
        h->async = as && std::strcmp(as, "0") != 0 && as[0] != '\0';
    }
    // fields, FP64 stage buffers and accumulators (FP64 path only), source; then the small tables
    const bool fp64_stage = p->precision != ATSAT_DYN_MIXED;
    const int64_t nbig = ATSAT_NFIELDS + (fp64_stage ? 2 * NPROG : 0) + 2;
    const int64_t nsmall = 2LL * K.im * 16 + K.im + K.jm + K.im + K.jm + 64;
    const size_t bytes = (size_t)(nbig * K.fsz + nsmall) * 8 + sizeof(ColGeo) * (size_t)K.im * K.jm + 4096;
    if ((e = cudaMalloc(&h->slab, bytes)) != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    if ((e = cudaMemsetAsync(h->slab, 0, bytes, h->stream)) != cudaSuccess) return cuda_fail(e, "cudaMemset");
    double* q = h->slab;
    for (int f = 0; f < ATSAT_NFIELDS; f++) { h->f[f] = q; q += K.fsz; }
    if (fp64_stage) {
        for (int s = 0; s < NPROG; s++) { h->stage[s] = q; q += K.fsz; }
        for (int s = 0; s < NPROG; s++) { h->acc[s] = q; q += K.fsz; }
    }
    h->src = q; q += K.fsz;
    h->p_baro = q; q += K.fsz;
    h->partial = q; q += 2LL * K.im * 16;
    h->buoy = q; q += K.im;
    h->sin_j = q; q += K.jm;
    h->rm_tab = q; q += K.im;
    h->cor_j = q; q += K.jm;
    h->counter = reinterpret_cast<unsigned long long*>(q);
    h->dev_err = reinterpret_cast<unsigned int*>(q + 1);
    q += 8;
    h->six = reinterpret_cast<double**>(q); q += 8;
    q = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(q) + 255) & ~uintptr_t(255));
    h->geo = reinterpret_cast<ColGeo*>(q);
    if (p->precision == ATSAT_DYN_MIXED) {
        // 118 arrays of fsz floats (the tensor maps' fourth dimension), then the two column tables
        h->n32 = 2 * NPROG + 2 + 3 * NPROG + 2 + NFZ + NCONV;
        const size_t ngeo = ((size_t)K.im * K.jm * (sizeof(ColGeoF) + sizeof(PrepGeo)) + 4095) / 4 + 1024;
        const size_t n32 = (size_t)h->n32 * K.fsz + ngeo;
        if ((e = cudaMalloc(&h->slab32, n32 * 4)) != cudaSuccess) return cuda_fail(e, "cudaMalloc (FP32)");
        if ((e = cudaMemsetAsync(h->slab32, 0, n32 * 4, h->stream)) != cudaSuccess) return cuda_fail(e, "cudaMemset");
        float* r = h->slab32;
        for (int s = 0; s < NPROG; s++) { h->yn32[s] = r; r += K.fsz; }
        h->wlo = r; r += K.fsz;
        for (int s = 0; s < NPROG; s++) { h->yo32[s] = r; r += K.fsz; }
        h->wlo_o = r; r += K.fsz;
        for (int s = 0; s < NPROG; s++) { h->dlA[s] = r; r += K.fsz; }
        for (int s = 0; s < NPROG; s++) { h->dlB[s] = r; r += K.fsz; }
        for (int s = 0; s < NPROG; s++) { h->dlC[s] = r; r += K.fsz; }
        h->edges_dirty = 0;
        for (int s = 0; s < 2; s++) { h->acc_turb[s] = r; r += K.fsz; }
        for (int s = 0; s < NFZ; s++) { h->fz[s] = r; r += K.fsz; }
        for (int s = 0; s < NCONV; s++) { h->conv32[s] = r; r += K.fsz; h->conv_dirty[s] = true; }
        if (r != h->slab32 + h->n32 * K.fsz) return fail(h, ATSAT_DYN_E_INVALID, "FP32 slab layout");
        r = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(r) + 255) & ~uintptr_t(255));
        h->geof = reinterpret_cast<ColGeoF*>(r);
        r += (size_t)K.im * K.jm * sizeof(ColGeoF) / 4;
        r = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(r) + 255) & ~uintptr_t(255));
        h->pgeo = reinterpret_cast<PrepGeo*>(r);
        if ((e = upload_geof(h)) != cudaSuccess) return cuda_fail(e, "FP32 geometry upload");
        h->tile_ok = make_tile_maps(h);
        h->march_levels = default_march_levels(h);
        // the default stage kernel: the fastest one measured at every grid tried, where it applies
        h->variant = variant_available(h, ATSAT_DYN_STAGE_MARCH) ? ATSAT_DYN_STAGE_MARCH
                   : (h->tile_ok ? ATSAT_DYN_STAGE_TILED : ATSAT_DYN_STAGE_DIRECT);
        // an earlier autotune of this configuration on this GPU model
        int cv = -1, cl = 0;
        if (tune_get(tune_cache_path(nullptr), K.im, K.jm, K.km, tune_knobs(h), device_name(h), &cv, &cl, nullptr) &&
            cv >= 0 && cv < ATSAT_DYN_STAGE_NVARIANT && variant_available(h, cv) && cl >= 1 && cl <= K.im - 2) {
            h->variant = cv;
            h->march_levels = cl;
            h->tuned_from_cache = true;
        }
    }
    // small host tables
    std::vector<double> sin_j(K.jm), rm_tab(K.im), cor_j(K.jm);
    const double nd = p->nd_cor ? p->L_atm * 1.0e3 / p->u_0 : 1.0;
    for (int j = 0; j < K.jm; j++) {
        sin_j[j] = std::sin(h->the_z[j]);
        cor_j[j] = p->coriolis_split ? p->Coriolis * nd * 2.0 * p->omega * std::fabs(std::sin(h->the_z[j])) : 0.0;
    }
    for (int i = 0; i < K.im; i++) rm_tab[i] = 1.0 / metric_radius(*p, h->rad_z[i]);
    double* six_h[6] = {h->f[ATSAT_F_AUX_U], h->f[ATSAT_F_AUX_V], h->f[ATSAT_F_AUX_W],
                        h->f[ATSAT_F_RHS_U], h->f[ATSAT_F_RHS_V], h->f[ATSAT_F_RHS_W]};
    if ((e = cudaMemcpyAsync(h->sin_j, sin_j.data(), 8 * K.jm, cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->rm_tab, rm_tab.data(), 8 * K.im, cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->cor_j, cor_j.data(), 8 * K.jm, cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->six, six_h, sizeof(six_h), cudaMemcpyHostToDevice, h->stream)) ||
        (e = cudaMemcpyAsync(h->geo, h->geo_h.data(), sizeof(ColGeo) * h->geo_h.size(), cudaMemcpyHostToDevice,
                             h->stream)) ||
        (e = cudaStreamSynchronize(h->stream)))
        return cuda_fail(e, "table upload");
    atsat_dyn_turb_params_default(&h->tp);
    if (p->turb_active) {
        *out = h;
        const int trc = setup_turbulence(h);
        if (trc) return trc;
    }
    if ((e = cudaMalloc(&h->clamp_added, (44 + clamp_partial_doubles()) * 8)) != cudaSuccess)
        return cuda_fail(e, "cudaMalloc (budget)");
    h->clamp_cells = reinterpret_cast<unsigned long long*>(h->clamp_added + 22);
    h->clamp_partial = h->clamp_added + 44;
    if ((e = cudaMemset(h->clamp_added, 0, 44 * 8)) != cudaSuccess) return cuda_fail(e, "cudaMemset (budget)");
    *out = h;
    return setup_press_variants(h);
}

void atsat_dyn_destroy(atsat_dyn_t h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& e : h->pend) { cudaEventDestroy(e.a); cudaEventDestroy(e.b); }
    for (auto e : h->pool) cudaEventDestroy(e);
    for (auto e : h->timer) if (e) cudaEventDestroy(e);
    poisson_destroy(h->poisson);
    if (h->pv_buf) cudaFree(h->pv_buf);
    if (h->clamp_added) cudaFree(h->clamp_added);
    if (h->turb_buf) cudaFree(h->turb_buf);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->slab) cudaFree(h->slab);
    if (h->slab32) cudaFree(h->slab32);
    for (int b = 0; b < 2; b++) {
        if (h->pinned[b]) cudaFreeHost(h->pinned[b]);
        if (h->ev_pin[b]) cudaEventDestroy(h->ev_pin[b]);
    }
    stage_pipe_free(h);
    for (int f = 0; f < ATSAT_NFIELDS; f++)
        if (h->dev_rows[f]) cudaFree(h->dev_rows[f]);
    if (h->astream) {
        cudaStreamSynchronize(h->astream);
        cudaStreamDestroy(h->astream);
    }
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_ajoin) cudaEventDestroy(h->ev_ajoin);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

const char* atsat_dyn_last_error(atsat_dyn_t h) { return h ? h->err.c_str() : "null handle"; }

int atsat_dyn_bind_host_rows(atsat_dyn_t h, int32_t field, double* const* rows) {
    if (!h || !h->slab) return ATSAT_DYN_E_INVALID;
    if (!valid_field(field) || !rows) return fail(h, ATSAT_DYN_E_INVALID, "bad field %d or rows", field);
    const size_t n = (size_t)h->kc.im * h->kc.jm;
    for (size_t r = 0; r < n; r++)
        if (!rows[r]) return fail(h, ATSAT_DYN_E_INVALID, "row %zu of field %d is null", r, field);
    h->bind_rows[field].assign(rows, rows + n);
    h->bind_kind[field] = BIND_ROWS;
    h->bind_base[field] = nullptr;
    return route_binding(h, field);
}

int atsat_dyn_bind_host_array(atsat_dyn_t h, int32_t field, double* base) {
    if (!h || !h->slab) return ATSAT_DYN_E_INVALID;
    if (!valid_field(field)) return fail(h, ATSAT_DYN_E_INVALID, "bad field %d", field);
    h->bind_kind[field] = base ? BIND_ARRAY : BIND_NONE;
    h->bind_base[field] = base;
    h->bind_rows[field].clear();
    return route_binding(h, field);
}

int atsat_dyn_set_host_direct(atsat_dyn_t h, int32_t enable) {
    if (!h || !h->slab || (enable != 0 && enable != 1)) return ATSAT_DYN_E_INVALID;
    if (enable && !h->host_ok)
        return fail(h, ATSAT_DYN_E_UNSUPPORTED, "the device does not address host memory through its page tables");
    CK(h, cudaSetDevice(h->device));
    h->host_direct = enable != 0;
    for (int f = 0; f < ATSAT_NFIELDS; f++)
        if (h->bind_kind[f] != BIND_NONE) {
            int rc = route_binding(h, f);
            if (rc) return rc;
        }
    return ATSAT_DYN_OK;
}

int atsat_dyn_host_direct(atsat_dyn_t h, int32_t field) {
    if (!h || !h->slab) return ATSAT_DYN_E_INVALID;
    if (field == -1) return h->host_direct ? 1 : 0;
    if (!valid_field(field)) return fail(h, ATSAT_DYN_E_INVALID, "bad field %d", field);
    return h->direct[field] ? 1 : 0;
}

int atsat_dyn_upload(atsat_dyn_t h, const int32_t* fields, int32_t n) {
    if (!h || !h->slab || (n > 0 && !fields)) return ATSAT_DYN_E_INVALID;
    CK(h, cudaSetDevice(h->device));
    bool n_level[NPROG] = {};
    bool prog = false;
    for (int32_t q = 0; q < n; q++) {
        if (fields[q] >= 0 && fields[q] < ATSAT_F_N_BASE + NPROG) prog = true;
        if (fields[q] >= ATSAT_F_N_BASE && fields[q] < ATSAT_F_N_BASE + NPROG && h->bind_kind[fields[q]] != BIND_NONE)
            n_level[fields[q] - ATSAT_F_N_BASE] = true;
    }
    if (prog) {
        int rc = unalias(h, n_level);
        if (rc) return rc;
    }
    HostBatch b{};
    for (int32_t q = 0; q < n; q++) {
        if (!valid_field(fields[q])) return fail(h, ATSAT_DYN_E_INVALID, "bad field %d", fields[q]);
        const int fid = fields[q];
        int rc = ATSAT_DYN_OK;
        if (h->direct[fid] && h->bind_kind[fid] != BIND_NONE) {
            mark_dirty(h, fid);
            rc = batch_add(h, b, fid, 1);
        } else {
            rc = upload_one(h, fid);
        }
        if (rc) return rc;
    }
    int rc = batch_flush(h, b, 1);
    if (!rc) rc = stage_join(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_download(atsat_dyn_t h, const int32_t* fields, int32_t n) {
    if (!h || !h->slab || (n > 0 && !fields)) return ATSAT_DYN_E_INVALID;
    CK(h, cudaSetDevice(h->device));
    HostBatch b{};
    for (int32_t q = 0; q < n; q++) {
        if (!valid_field(fields[q])) return fail(h, ATSAT_DYN_E_INVALID, "bad field %d", fields[q]);
        const int fid = fields[q];
        const int rc = (h->direct[fid] && h->bind_kind[fid] != BIND_NONE) ? batch_add(h, b, fid, 0)
                                                                          : download_one(h, fid);
        if (rc) { h->rows_pending = -1; return rc; }
    }
    int rc = batch_flush(h, b, 0);
    if (!rc) rc = rows_flush(h);
    if (!rc) rc = stage_join(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_set_tables(atsat_dyn_t h, const double* cell_vbar0, const double* cell_ubar0, const double* p_baro) {
    if (!h || !h->slab) return ATSAT_DYN_E_INVALID;
    if ((cell_vbar0 == nullptr) != (cell_ubar0 == nullptr))
        return fail(h, ATSAT_DYN_E_INVALID, "cell_vbar0 and cell_ubar0 must both be given or both be null");
    CK(h, cudaSetDevice(h->device));
    build_geometry(h, cell_vbar0, cell_ubar0);
    CK(h, cudaMemcpyAsync(h->geo, h->geo_h.data(), sizeof(ColGeo) * h->geo_h.size(), cudaMemcpyHostToDevice,
                          h->stream));
    if (h->geof) CK(h, upload_geof(h));
    h->has_pbaro = (p_baro != nullptr);
    if (p_baro) {
        const KConst& K = h->kc;
        CK(h, cudaMemcpy2DAsync(h->p_baro, (size_t)K.kp * 8, p_baro, (size_t)K.km * 8, (size_t)K.km * 8,
                                (size_t)K.im * K.jm, cudaMemcpyHostToDevice, h->stream));
    }
    return finish(h);
}

int atsat_dyn_get_buoy_ref_level(atsat_dyn_t h, double* out) {
    if (!h || !h->slab || !out) return ATSAT_DYN_E_INVALID;
    CK(h, cudaSetDevice(h->device));
    CK(h, cudaMemcpyAsync(out, h->buoy, 8 * (size_t)h->kc.im, cudaMemcpyDeviceToHost, h->stream));
    return finish(h, true);
}

#define ENTRY(h)                                              \
    if (!h || !h->slab) return ATSAT_DYN_E_INVALID;           \
    CK(h, cudaSetDevice(h->device))

int atsat_dyn_mixture_density(atsat_dyn_t h) {
    ENTRY(h);
    {
        Timed t(h, ATSAT_K_GLUE);
        CK(h, launch_density(h->kc, h->f[ATSAT_F_T], h->f[ATSAT_F_P_STAT], h->p.R_mix, h->f[ATSAT_F_RHO_MIX], h->stream));
        h->launches += 1;
        mark_dirty(h, ATSAT_F_RHO_MIX);
    }
    return finish(h);
}

int atsat_dyn_buoyancy_ref_level(atsat_dyn_t h) {
    ENTRY(h);
    int rc = do_level_mean(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_metric_pressure(atsat_dyn_t h) {
    ENTRY(h);
    int rc = do_metric(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_rhs(atsat_dyn_t h) {
    ENTRY(h);
    { int rc0 = unalias(h); if (rc0) return rc0; }
    double* L[NPROG];
    for (int q = 0; q < NPROG; q++) L[q] = h->f[q];
    if (h->p.precision == ATSAT_DYN_MIXED) {
        int rc = enqueue_mixed_prepare(h, L, 0u, false);   // the stencils read the live fields
        if (rc) return rc;
        MixedIO io = make_mixed_io(h, nullptr, nullptr, nullptr);
        for (int q = 0; q < NPROG; q++) io.yn64[q] = L[q];
        StageParams sp{};
        {
            Timed t(h, ATSAT_K_RHS);
            CK(h, launch_rk_stage_mixed(h->kf, io, sp, MODE_RHS, h->stream));
            h->launches += 1;
        }
        return finish(h);
    }
    StageIO<double> io = make_io(h, L, nullptr);
    StageParams sp{};
    {
        Timed t(h, ATSAT_K_RHS);
        CK(h, launch_rk_stage_fp64(h->kc, io, sp, MODE_RHS, h->stream));
        h->launches += 1;
    }
    return finish(h);
}

int atsat_dyn_rk4_step(atsat_dyn_t h) {
    ENTRY(h);
    { int rc0 = unalias(h); if (rc0) return rc0; }
    int rc = enqueue_rk4(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_prepare_projection_boundaries(atsat_dyn_t h) {
    ENTRY(h);
    {
        Timed t(h, ATSAT_K_PRESS_BOUNDARY);
        CK(h, launch_projection_prep(h->kc, h->six, h->stream));
        h->launches += 2;
    }
    return finish(h);
}

int atsat_dyn_pressure(atsat_dyn_t h, atsat_dyn_pstats* out) {
    ENTRY(h);
    const int sweeps = h->p.press_sweeps > 0 ? h->p.press_sweeps : 1;
    int rc = enqueue_pressure(h, sweeps);
    if (rc) return rc;
    rc = finish(h, out != nullptr);
    if (rc) return rc;
    if (out) {
        unsigned long long n = 0;
        CK(h, cudaMemcpy(&n, h->counter, sizeof(n), cudaMemcpyDeviceToHost));
        out->sweeps = sweeps;
        out->src_clamped = (double)n;
        out->max_abs_update = -1.0;      // not tracked on the device
    }
    return ATSAT_DYN_OK;
}

int atsat_dyn_restore_var(atsat_dyn_t h) {
    ENTRY(h);
    { int rc0 = unalias(h); if (rc0) return rc0; }
    int rc = enqueue_restore(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_boundary_conditions(atsat_dyn_t h) {
    ENTRY(h);
    { int rc0 = unalias(h); if (rc0) return rc0; }
    int rc = enqueue_bc(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_damp_wiggles(atsat_dyn_t h, int32_t field, int32_t along_i, int32_t along_j, int32_t along_k,
                           double strength, int32_t passes) {
    ENTRY(h);
    if (!valid_field(field) || passes < 0) return fail(h, ATSAT_DYN_E_INVALID, "damp_wiggles: bad field or passes");
    { int rc0 = unalias(h); if (rc0) return rc0; }
    int rc = enqueue_damp(h, field, along_i != 0, along_j != 0, along_k != 0, strength, passes);
    return rc ? rc : finish(h);
}

int atsat_dyn_damp_pdyn(atsat_dyn_t h) {
    ENTRY(h);
    int rc = enqueue_damp_pdyn(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_clamp_negative_species(atsat_dyn_t h) {
    ENTRY(h);
    { int rc0 = unalias(h); if (rc0) return rc0; }
    int rc = enqueue_clamp(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_turb_params_default(atsat_dyn_turb_params* tp) {
    if (!tp) return ATSAT_DYN_E_INVALID;
    *tp = atsat_dyn_turb_params{};
    tp->model = ATSAT_TURB_K_OMEGA_SST; tp->turb_free = 1; tp->clamp_pass = 1; tp->abl_taper = 0; tp->curv = 1;
    tp->buoy = 3;                                  // cSaturnModel::turb_default_buoy() (cSaturnModel.h:299)
    tp->k_bg = 1.0; tp->l_bg = 0.0; tp->nue_max_phys = 1.0e5; tp->vel_star_max = std::sqrt(0.002) * 200.0;
    tp->vel_star_ref = 0.4; tp->z_0 = 0.1; tp->nue_gas = 1.8e-5;       // TurbulenceSat's constructor defaults
    tp->abl_height = 20000.0;                                          // cSaturnModel.h:1281
    // H2O, NH3, CH4: the moist gases of cSaturnModel::moist_gas_for_turb (cSaturnModel.cpp:259-266), values
    // read back from the reference's build
    const double ep[3] = {8.1253, 7.6752, 7.6752}, lv[3] = {2.5009e6, 1.372e6, 5.11e5};
    const double ls[3] = {2.8339e6, 1.832e6, 5.11e5}, t0[3] = {273.15, 195.5, 90.69};
    for (int n = 0; n < 3; n++) { tp->ep[n] = ep[n]; tp->lv[n] = lv[n]; tp->ls[n] = ls[n]; tp->t_0[n] = t0[n]; }
    return ATSAT_DYN_OK;
}

int atsat_dyn_turb_params_from_env(atsat_dyn_turb_params* tp) {
    if (!tp) return ATSAT_DYN_E_INVALID;
    if (const char* e = getenv("ATSAT_TURB_MODEL")) {
        const std::string m(e);
        tp->model = m == "k_epsilon" ? ATSAT_TURB_K_EPSILON : (m == "k_omega" ? ATSAT_TURB_K_OMEGA : ATSAT_TURB_K_OMEGA_SST);
    }
    if (const char* e = getenv("ATSAT_TURB_FREE")) tp->turb_free = atoi(e);
    if (const char* e = getenv("ATSAT_TURB_CLAMP_PASS")) tp->clamp_pass = atoi(e);
    if (const char* e = getenv("ATSAT_ABL_TAPER")) tp->abl_taper = atoi(e);
    if (const char* e = getenv("ATSAT_TURB_CURV")) tp->curv = atoi(e) != 0;
    if (const char* e = getenv("ATSAT_TURB_BUOY")) tp->buoy = atoi(e);
    if (const char* e = getenv("ATSAT_TURB_K_BG")) tp->k_bg = atof(e);
    if (const char* e = getenv("ATSAT_TURB_L_BG")) tp->l_bg = atof(e);
    if (const char* e = getenv("ATSAT_NUE_MAX")) tp->nue_max_phys = atof(e);
    if (const char* e = getenv("ATSAT_VEL_STAR_MAX")) tp->vel_star_max = atof(e);
    return ATSAT_DYN_OK;
}

int atsat_dyn_set_turb_params(atsat_dyn_t h, const atsat_dyn_turb_params* tp) {
    if (!h || !h->slab || !tp) return ATSAT_DYN_E_INVALID;
    if (tp->model < ATSAT_TURB_K_EPSILON || tp->model > ATSAT_TURB_K_OMEGA_SST)
        return fail(h, ATSAT_DYN_E_INVALID, "turbulence: unknown model %d", tp->model);
    if (!tp->clamp_pass)
        return fail(h, ATSAT_DYN_E_UNSUPPORTED, "ATSAT_TURB_CLAMP_PASS=0: the reference's sources then read neighbours "
                    "other threads are flooring, so its result depends on the thread count (Turbulence.h:165-173)");
    h->tp = *tp;
    return ATSAT_DYN_OK;
}

int atsat_dyn_turbulence(atsat_dyn_t h) {
    ENTRY(h);
    { int rc0 = unalias(h); if (rc0) return rc0; }
    int rc = enqueue_turbulence(h);
    return rc ? rc : finish(h);
}

int atsat_dyn_turbulence_diag(atsat_dyn_t h, double* prod, double* vel_star) {
    ENTRY(h);
    if (!h->turb_buf) return fail(h, ATSAT_DYN_E_INVALID, "turbulence_diag: the closure has not run");
    const KConst& K = h->kc;
    CK(h, cudaStreamSynchronize(h->stream));
    if (prod)
        CK(h, cudaMemcpy2D(prod, (size_t)K.km * 8, h->turb_prod, (size_t)K.kp * 8, (size_t)K.km * 8,
                           (size_t)K.im * K.jm, cudaMemcpyDeviceToHost));
    if (vel_star)
        CK(h, cudaMemcpy2D(vel_star, (size_t)K.km * 8, h->turb_vs, (size_t)K.kp * 8, (size_t)K.km * 8, (size_t)K.jm,
                           cudaMemcpyDeviceToHost));
    return ATSAT_DYN_OK;
}

}  // extern "C"

namespace {

// cSaturnModel::restart_arrays and restart_arrays_carried (FileIO_Sat.cpp:513-552), in file order: a device
// field id, or -1 - n for the caller's host array n. The carried list's last entry (S_precip_ch4) is SAT3 only.
const int RESTART_MAIN[38] = {
    ATSAT_F_T, ATSAT_F_U, ATSAT_F_V, ATSAT_F_W, ATSAT_F_TN, ATSAT_F_UN, ATSAT_F_VN, ATSAT_F_WN,
    ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2ON, ATSAT_F_H2O_CLOUDN, ATSAT_F_H2O_ICEN,
    ATSAT_F_H2S, ATSAT_F_H2SN,
    ATSAT_F_NH3, ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_NH3N, ATSAT_F_NH3_CLOUDN, ATSAT_F_NH3_ICEN,
    ATSAT_F_CH4, ATSAT_F_CH4_CLOUD, ATSAT_F_CH4_ICE, ATSAT_F_CH4N, ATSAT_F_CH4_CLOUDN, ATSAT_F_CH4_ICEN,
    ATSAT_F_NH4SH, ATSAT_F_NH4SHN,
    ATSAT_F_P_DYN, ATSAT_F_P_DYNN, ATSAT_F_P_STAT,
    ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_TKEN, ATSAT_F_DISN, ATSAT_F_NUE};
const int RESTART_CARRIED[35] = {
    ATSAT_F_TKE_SOURCE, ATSAT_F_DIS_SOURCE,
    -1, -2, -3,                                          // difflux_h2s, _nh3, _nh4sh
    -4, -5, -6,                                          // j_h2s, _nh3, _nh4sh
    ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH,
    ATSAT_F_THERMALMASSFLUX, ATSAT_F_FLUXLIM_NH4SH,
    ATSAT_F_RHS_U, ATSAT_F_RHS_V,
    ATSAT_F_RHO_MIX, ATSAT_F_Q_PRECIP,
    ATSAT_F_S_PRECIP_H2O, ATSAT_F_S_PRECIP_H2O_CLOUD, ATSAT_F_S_PRECIP_H2O_ICE,
    ATSAT_F_S_PRECIP_NH3, ATSAT_F_S_PRECIP_NH3_ICE,
    ATSAT_F_S_PRECIP_NH3_CLOUD, ATSAT_F_S_PRECIP_CH4_CLOUD, ATSAT_F_S_PRECIP_CH4_ICE,
    -7, -8, -9,                                          // w_h2s, _nh3, _nh4sh
    -10, -11, -12, -13, -14, -15,                        // BuoyancyForce, PresGradForce, Q_Sensible, jT_*
    ATSAT_F_S_PRECIP_CH4};
constexpr int32_t MAGIC_SAT1 = 0x53415431, MAGIC_SAT2 = 0x53415432, MAGIC_SAT3 = 0x53415433;

std::vector<int> restart_list(int format) {
    std::vector<int> v(RESTART_MAIN, RESTART_MAIN + 38);
    if (format >= 2) v.insert(v.end(), RESTART_CARRIED, RESTART_CARRIED + (format == 3 ? 35 : 34));
    return v;
}

// two pinned buffers of im*jm*km doubles for the restart streams, allocated on first use
int restart_buffers(atsat_dyn* h, double** buf) {
    static_assert(sizeof(double) == 8, "double");
    const size_t bytes = (size_t)h->kc.im * h->kc.jm * h->kc.km * 8;
    for (int b = 0; b < 2; b++) {
        const cudaError_t e = cudaHostAlloc(&buf[b], bytes, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            if (b) cudaFreeHost(buf[0]);
            return fail(h, ATSAT_DYN_E_NOMEM, "restart staging: %s", cudaGetErrorString(e));
        }
    }
    return ATSAT_DYN_OK;
}

}  // namespace

extern "C" {

int atsat_dyn_save_restart(atsat_dyn_t h, const char* path, int32_t iter, int32_t carried,
                           const double* const* host_arrays) {
    ENTRY(h);
    if (!path) return fail(h, ATSAT_DYN_E_INVALID, "save_restart: null path");
    const KConst& K = h->kc;
    const size_t n = (size_t)K.im * K.jm * K.km;
    FILE* f = fopen(path, "wb");
    if (!f) return fail(h, ATSAT_DYN_E_INVALID, "save_restart: cannot open %s", path);
    const int32_t hdr[5] = {carried ? MAGIC_SAT3 : MAGIC_SAT1, K.im, K.jm, K.km, iter};
    bool ok = fwrite(hdr, sizeof(hdr), 1, f) == 1;
    double* buf[2] = {nullptr, nullptr};
    int rc = restart_buffers(h, buf);
    if (rc) { fclose(f); return rc; }
    cudaEvent_t ev[2];
    cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    std::vector<double> zeros;
    const std::vector<int> list = restart_list(carried ? 3 : 1);
    // device field q: a pitched-to-contiguous copy into buffer q & 1 while the previous one is written out
    auto fetch = [&](size_t q) -> cudaError_t {
        const int id = list[q];
        if (id < 0) return cudaSuccess;
        const int b = (int)(q & 1);
        cudaError_t e = cudaMemcpy2DAsync(buf[b], (size_t)K.km * 8, h->f[id], (size_t)K.kp * 8, (size_t)K.km * 8,
                                          (size_t)K.im * K.jm, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaEventRecord(ev[b], h->stream);
        return e;
    };
    cudaError_t e = list.empty() ? cudaSuccess : fetch(0);
    for (size_t q = 0; q < list.size() && ok && e == cudaSuccess; q++) {
        if (q + 1 < list.size()) e = fetch(q + 1);
        if (e != cudaSuccess) break;
        const int id = list[q];
        const double* src;
        if (id >= 0) {
            e = cudaEventSynchronize(ev[q & 1]);
            src = buf[q & 1];
        } else {
            src = host_arrays ? host_arrays[-1 - id] : nullptr;
            if (!src) {
                if (zeros.empty()) zeros.assign(n, 0.0);
                src = zeros.data();
            }
        }
        ok = e == cudaSuccess && fwrite(src, 8, n, f) == n;
    }
    cudaStreamSynchronize(h->stream);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaFreeHost(buf[0]);
    cudaFreeHost(buf[1]);
    ok = (fclose(f) == 0) && ok;
    if (e != cudaSuccess) return fail(h, ATSAT_DYN_E_CUDA, "save_restart: %s", cudaGetErrorString(e));
    if (!ok) return fail(h, ATSAT_DYN_E_INVALID, "save_restart: write failed on %s (disk full?)", path);
    return ATSAT_DYN_OK;
}

int atsat_dyn_load_restart(atsat_dyn_t h, const char* path, int32_t* iter, int32_t* format, double* const* host_arrays) {
    ENTRY(h);
    if (!path) return fail(h, ATSAT_DYN_E_INVALID, "load_restart: null path");
    const KConst& K = h->kc;
    const size_t n = (size_t)K.im * K.jm * K.km;
    FILE* f = fopen(path, "rb");
    if (!f) return fail(h, ATSAT_DYN_E_INVALID, "load_restart: no file %s", path);
    int32_t hdr[5];
    const bool got = fread(hdr, sizeof(hdr), 1, f) == 1;
    const int fmt = !got ? 0 : hdr[0] == MAGIC_SAT3 ? 3 : hdr[0] == MAGIC_SAT2 ? 2 : hdr[0] == MAGIC_SAT1 ? 1 : 0;
    if (!fmt || hdr[1] != K.im || hdr[2] != K.jm || hdr[3] != K.km) {
        fclose(f);
        return fail(h, ATSAT_DYN_E_INVALID, "load_restart: bad header / grid mismatch in %s", path);
    }
    { int rc0 = unalias(h); if (rc0) { fclose(f); return rc0; } }
    double* buf[2] = {nullptr, nullptr};
    int rc = restart_buffers(h, buf);
    if (rc) { fclose(f); return rc; }
    cudaEvent_t ev[2];
    cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    bool recorded[2] = {false, false};
    const std::vector<int> list = restart_list(fmt);
    bool ok = true;
    cudaError_t e = cudaSuccess;
    for (size_t q = 0; q < list.size() && ok && e == cudaSuccess; q++) {
        const int id = list[q];
        if (id >= 0) {
            const int b = (int)(q & 1);
            if (recorded[b]) e = cudaEventSynchronize(ev[b]);      // the buffer's previous upload is done
            if (e != cudaSuccess) break;
            ok = fread(buf[b], 8, n, f) == n;
            if (!ok) break;
            e = cudaMemcpy2DAsync(h->f[id], (size_t)K.kp * 8, buf[b], (size_t)K.km * 8, (size_t)K.km * 8,
                                  (size_t)K.im * K.jm, cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess) e = cudaEventRecord(ev[b], h->stream);
            recorded[b] = true;
            mark_dirty(h, id);
        } else {
            double* dst = host_arrays ? host_arrays[-1 - id] : nullptr;
            ok = dst ? fread(dst, 8, n, f) == n : fseek(f, (long)(n * 8), SEEK_CUR) == 0;
        }
    }
    cudaStreamSynchronize(h->stream);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaFreeHost(buf[0]);
    cudaFreeHost(buf[1]);
    fclose(f);
    if (e != cudaSuccess) return fail(h, ATSAT_DYN_E_CUDA, "load_restart: %s", cudaGetErrorString(e));
    if (!ok) return fail(h, ATSAT_DYN_E_INVALID, "load_restart: truncated file %s", path);
    if (iter) *iter = hdr[4];
    if (format) *format = fmt;
    return finish(h, true);
}

int atsat_dyn_restart_is_clean(atsat_dyn_t h, int32_t* clean) {
    ENTRY(h);
    if (!clean) return fail(h, ATSAT_DYN_E_INVALID, "restart_is_clean: null output");
    const double* fl[38];
    for (int q = 0; q < 38; q++) fl[q] = h->f[RESTART_MAIN[q]];
    CK(h, cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), h->stream));
    CK(h, launch_nonfinite_fields(h->kc, fl, 38, h->counter, h->stream));
    h->launches += 1;
    unsigned long long c = 0;
    CK(h, cudaMemcpyAsync(&c, h->counter, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
    int rc = finish(h, true);
    if (rc) return rc;
    *clean = c == 0 ? 1 : 0;
    return ATSAT_DYN_OK;
}

int atsat_dyn_clamp_budget(atsat_dyn_t h, double* added, int64_t* cells, double* added_bnd, int64_t* cells_bnd) {
    ENTRY(h);
    if (!added || !cells || !added_bnd || !cells_bnd) return fail(h, ATSAT_DYN_E_INVALID, "clamp_budget: null output");
    double a[22];
    unsigned long long c[22];
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaMemcpy(a, h->clamp_added, sizeof(a), cudaMemcpyDeviceToHost));
    CK(h, cudaMemcpy(c, h->clamp_cells, sizeof(c), cudaMemcpyDeviceToHost));
    for (int q = 0; q < 11; q++) {
        added[q] = a[q];
        added_bnd[q] = a[11 + q];
        cells[q] = (int64_t)c[q];
        cells_bnd[q] = (int64_t)c[11 + q];
    }
    return ATSAT_DYN_OK;
}

}  // extern "C"

namespace {

// one resident dycore iteration (cSaturnModel.cpp:864-1111 restricted to the dycore), enqueued
int enqueue_iteration(atsat_dyn* h, int32_t it) {
    int rc;
    if (it % 2 == 0 || h->p.press_every_step) {
        {
            Timed t(h, ATSAT_K_GLUE);
            CK(h, launch_density(h->kc, h->f[ATSAT_F_T], h->f[ATSAT_F_P_STAT], h->p.R_mix, h->f[ATSAT_F_RHO_MIX],
                                 h->stream));
            h->launches += 1;
            mark_dirty(h, ATSAT_F_RHO_MIX);
        }
        if ((rc = enqueue_pressure(h, h->p.press_sweeps > 0 ? h->p.press_sweeps : 1))) return rc;
        if (h->p.driver_glue && (rc = enqueue_damp_pdyn(h))) return rc;
    }
    if ((rc = enqueue_rk4(h, true))) return rc;
    if ((rc = enqueue_bc(h, true))) return rc;
    if (h->p.driver_glue && (rc = enqueue_clamp(h, true))) return rc;
    if ((rc = enqueue_restore(h, true))) return rc;
    if (h->p.driver_glue && h->p.turb_active && (rc = enqueue_turbulence(h, true))) return rc;
    return ATSAT_DYN_OK;
}

bool resident_steady(const atsat_dyn* h) {
    if (h->p.precision != ATSAT_DYN_MIXED) return true;
    if (!(h->aliased && h->shadow_valid && h->edges_dirty == 0 && h->split_mask == 0)) return false;
    for (int s = 0; s < NCONV; s++)
        if (h->conv_dirty[s]) return false;
    return true;
}

}  // namespace

extern "C" {

int atsat_dyn_iterate(atsat_dyn_t h, int32_t iter0, int32_t n) {
    ENTRY(h);
    if (n < 0) return fail(h, ATSAT_DYN_E_INVALID, "negative iteration count");
    for (int32_t it = iter0; it < iter0 + n; it++) {
        const int rc = enqueue_iteration(h, it);
        if (rc) return rc;
    }
    return finish(h);
}

int atsat_dyn_graph_capture(atsat_dyn_t h, int32_t iter0, int32_t n) {
    ENTRY(h);
    if (n < 2 || (n & 1)) return fail(h, ATSAT_DYN_E_INVALID, "graph_capture: n must be even and >= 2");
    if (!resident_steady(h))
        return fail(h, ATSAT_DYN_E_INVALID, "graph_capture: run two resident iterations first (the mixed path's "
                    "resident buffers are not established yet)");
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    const bool prof = h->profiling;
    h->profiling = false;
    const int64_t l0 = h->launches;
    cudaGraph_t g = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = ATSAT_DYN_OK;
    for (int32_t it = iter0; it < iter0 + n && rc == ATSAT_DYN_OK; it++) rc = enqueue_iteration(h, it);
    const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    h->profiling = prof;
    h->graph_kernels = h->launches - l0;
    h->launches = l0;                                  // captured, not run
    if (rc != ATSAT_DYN_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return fail(h, ATSAT_DYN_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
    // n is even: the FP32 copies swapped back to where they were; the steady flags still hold
    if (!resident_steady(h)) { cudaGraphDestroy(g); return fail(h, ATSAT_DYN_E_INVALID, "graph_capture: state moved"); }
    const cudaError_t ei = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) { h->graph = nullptr; return fail(h, ATSAT_DYN_E_CUDA, "graph instantiate: %s", cudaGetErrorString(ei)); }
    h->graph_iters = n;
    return ATSAT_DYN_OK;
}

int atsat_dyn_graph_launch(atsat_dyn_t h, int32_t reps) {
    ENTRY(h);
    if (!h->graph || reps < 0) return fail(h, ATSAT_DYN_E_INVALID, "graph_launch: no captured graph");
    for (int32_t r = 0; r < reps; r++) CK(h, cudaGraphLaunch(h->graph, h->stream));
    h->launches += (int64_t)reps * h->graph_kernels;
    return ATSAT_DYN_OK;
}

int atsat_dyn_ensemble_run(const atsat_dyn_t* members, int32_t n, int32_t reps, int32_t concurrent, double* ms) {
    if (!members || n < 1 || reps < 0 || !ms) return ATSAT_DYN_E_INVALID;
    for (int32_t m = 0; m < n; m++)
        if (!members[m] || !members[m]->graph) return ATSAT_DYN_E_INVALID;
    atsat_dyn* h0 = members[0];
    std::vector<cudaEvent_t> done(n);
    cudaEvent_t start, stop;
    CK(h0, cudaEventCreate(&start));
    CK(h0, cudaEventCreate(&stop));
    for (int32_t m = 0; m < n; m++) CK(h0, cudaEventCreateWithFlags(&done[m], cudaEventDisableTiming));
    CK(h0, cudaEventRecord(start, h0->stream));
    for (int32_t m = 0; m < n; m++) {
        atsat_dyn* h = members[m];
        // every member starts after `start`; one after another: also after the previous member
        CK(h0, cudaStreamWaitEvent(h->stream, (concurrent || m == 0) ? start : done[m - 1], 0));
        if (concurrent) continue;
        for (int32_t r = 0; r < reps; r++) CK(h0, cudaGraphLaunch(h->graph, h->stream));
        h->launches += (int64_t)reps * h->graph_kernels;
        CK(h0, cudaEventRecord(done[m], h->stream));
    }
    if (concurrent) {
        // round-robin over the members so that every stream has work queued early
        for (int32_t r = 0; r < reps; r++)
            for (int32_t m = 0; m < n; m++) CK(h0, cudaGraphLaunch(members[m]->graph, members[m]->stream));
        for (int32_t m = 0; m < n; m++) {
            members[m]->launches += (int64_t)reps * members[m]->graph_kernels;
            CK(h0, cudaEventRecord(done[m], members[m]->stream));
        }
    }
    for (int32_t m = 0; m < n; m++) CK(h0, cudaStreamWaitEvent(h0->stream, done[m], 0));
    CK(h0, cudaEventRecord(stop, h0->stream));
    CK(h0, cudaEventSynchronize(stop));
    float t = 0.0f;
    CK(h0, cudaEventElapsedTime(&t, start, stop));
    *ms = t;
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    for (auto e : done) cudaEventDestroy(e);
    for (int32_t m = 0; m < n; m++) {
        const int rc = finish(members[m]);
        if (rc) return rc;
    }
    return ATSAT_DYN_OK;
}

int atsat_dyn_sync(atsat_dyn_t h) {
    ENTRY(h);
    return finish(h, true);
}

int atsat_dyn_set_async(atsat_dyn_t h, int32_t enable) {
    if (!h || !h->slab || (enable != 0 && enable != 1)) return ATSAT_DYN_E_INVALID;
    if (h->async && !enable) {
        int rc = finish(h, true);
        h->async = false;
        return rc;
    }
    h->async = enable != 0;
    return ATSAT_DYN_OK;
}

int atsat_dyn_set_wait_test(atsat_dyn_t h, int64_t clocks, int32_t withhold) {
    if (!h) return ATSAT_DYN_E_INVALID;
    if (clocks < 0 || clocks > TILE_WAIT_LIMIT || withhold < 0 || withhold > 8)
        return fail(h, ATSAT_DYN_E_INVALID, "set_wait_test: clocks in [0, 2^31] (0: default), withhold in [0, 8]");
    h->wait_limit = clocks ? clocks : TILE_WAIT_LIMIT;
    h->test_withhold = withhold;
    return ATSAT_DYN_OK;
}

int atsat_dyn_status(atsat_dyn_t h, atsat_dyn_diag* out) {
    if (!h || !out) return ATSAT_DYN_E_INVALID;
    memset(out, 0, sizeof(*out));
    out->launches = h->launches;
    out->timeout = h->timeouts;
    out->tuned_from_cache = h->tuned_from_cache ? 1 : 0;
    return ATSAT_DYN_OK;
}

int atsat_dyn_count_nonfinite(atsat_dyn_t h, int32_t field, int64_t* count) {
    ENTRY(h);
    if (!valid_field(field) || !count) return fail(h, ATSAT_DYN_E_INVALID, "bad field %d", field);
    CK(h, cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), h->stream));
    CK(h, launch_count_nonfinite(h->kc, h->f[field], h->counter, h->stream));
    h->launches += 1;
    unsigned long long n = 0;
    CK(h, cudaMemcpyAsync(&n, h->counter, sizeof(n), cudaMemcpyDeviceToHost, h->stream));
    int rc = finish(h, true);
    *count = (int64_t)n;
    return rc;
}

int atsat_dyn_profile(atsat_dyn_t h, int32_t enable) {
    if (!h) return ATSAT_DYN_E_INVALID;
    int rc = resolve_profile(h);
    h->profiling = enable != 0;
    h->prof_mask = ~0u;
    return rc;
}

int atsat_dyn_profile_classes(atsat_dyn_t h, uint32_t mask) {
    if (!h) return ATSAT_DYN_E_INVALID;
    int rc = resolve_profile(h);
    h->profiling = mask != 0;
    h->prof_mask = mask;
    return rc;
}

int atsat_dyn_profile_reset(atsat_dyn_t h) {
    if (!h) return ATSAT_DYN_E_INVALID;
    int rc = resolve_profile(h);
    for (int c = 0; c < ATSAT_K_NCLASS; c++) { h->prof_n[c] = 0; h->prof_ms[c] = 0.0; }
    return rc;
}

int atsat_dyn_profile_read(atsat_dyn_t h, int32_t kclass, int64_t* launches, double* ms) {
    if (!h || kclass < 0 || kclass >= ATSAT_K_NCLASS) return ATSAT_DYN_E_INVALID;
    int rc = resolve_profile(h);
    if (launches) *launches = h->prof_n[kclass];
    if (ms) *ms = h->prof_ms[kclass];
    return rc;
}

int atsat_dyn_timer_start(atsat_dyn_t h) {
    ENTRY(h);
    if (!h->timer[0]) {
        CK(h, cudaEventCreate(&h->timer[0]));
        CK(h, cudaEventCreate(&h->timer[1]));
    }
    CK(h, cudaEventRecord(h->timer[0], h->stream));
    return ATSAT_DYN_OK;
}

int atsat_dyn_timer_stop(atsat_dyn_t h, double* ms) {
    ENTRY(h);
    if (!h->timer[0] || !ms) return fail(h, ATSAT_DYN_E_INVALID, "timer_stop without timer_start");
    CK(h, cudaEventRecord(h->timer[1], h->stream));
    CK(h, cudaEventSynchronize(h->timer[1]));
    float f = 0.f;
    CK(h, cudaEventElapsedTime(&f, h->timer[0], h->timer[1]));
    *ms = f;
    return ATSAT_DYN_OK;
}

int atsat_dyn_device_field(atsat_dyn_t h, int32_t field, double** dptr, int64_t* pitch) {
    if (!h || !h->slab || !valid_field(field)) return ATSAT_DYN_E_INVALID;
    if (dptr) *dptr = h->f[field];
    if (pitch) *pitch = h->kc.kp;
    return ATSAT_DYN_OK;
}

void* atsat_dyn_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
}

void atsat_dyn_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

// test hook: write every rhs_* at the last RK stage, as RHSSat does at every stage
int atsat_dyn_set_write_all_rhs(atsat_dyn_t h, int32_t on) {
    if (!h) return ATSAT_DYN_E_INVALID;
    h->write_all_rhs = on != 0;
    return ATSAT_DYN_OK;
}

int atsat_dyn_set_stage_variant(atsat_dyn_t h, int32_t variant) {
    if (!h) return ATSAT_DYN_E_INVALID;
    if (variant < 0 || variant >= ATSAT_DYN_STAGE_NVARIANT)
        return fail(h, ATSAT_DYN_E_INVALID, "unknown stage variant %d", variant);
    if (h->p.precision != ATSAT_DYN_MIXED)
        return fail(h, ATSAT_DYN_E_UNSUPPORTED, "stage variants are a mixed-precision setting");
    if (!variant_available(h, variant))
        return fail(h, ATSAT_DYN_E_UNSUPPORTED, "stage variant %d unavailable here (tiled: no tensor-map encoder; "
                    "split: species_divu on)", variant);
    h->variant = variant;
    return ATSAT_DYN_OK;
}

int atsat_dyn_tune_cache_get(const char* path, int32_t im, int32_t jm, int32_t km, uint32_t knobs, const char* gpu,
                             int32_t* variant, int32_t* levels, double* ms) {
    if (!variant || !levels) return ATSAT_DYN_E_INVALID;
    int v = -1, l = 0;
    if (!tune_get(tune_cache_path(path), im, jm, km, knobs, tune_gpu_token(gpu), &v, &l, ms)) return ATSAT_DYN_E_INVALID;
    *variant = v;
    *levels = l;
    return ATSAT_DYN_OK;
}

int atsat_dyn_tune_cache_put(const char* path, int32_t im, int32_t jm, int32_t km, uint32_t knobs, const char* gpu,
                             int32_t variant, int32_t levels, double ms) {
    if (variant < 0 || variant >= ATSAT_DYN_STAGE_NVARIANT || levels < 1) return ATSAT_DYN_E_INVALID;
    return tune_put(tune_cache_path(path), im, jm, km, knobs, tune_gpu_token(gpu), variant, levels, ms)
               ? ATSAT_DYN_OK : ATSAT_DYN_E_INVALID;
}

int atsat_dyn_set_march_levels(atsat_dyn_t h, int32_t levels) {
    if (!h) return ATSAT_DYN_E_INVALID;
    if (levels < 1 || levels > h->kc.im - 2)
        return fail(h, ATSAT_DYN_E_INVALID, "march levels %d outside 1 .. im-2 = %d", levels, h->kc.im - 2);
    h->march_levels = levels;
    return ATSAT_DYN_OK;
}

int atsat_dyn_get_march_levels(atsat_dyn_t h, int32_t* levels) {
    if (!h || !levels) return ATSAT_DYN_E_INVALID;
    *levels = h->march_levels;
    return ATSAT_DYN_OK;
}

int atsat_dyn_get_stage_variant(atsat_dyn_t h, int32_t* variant) {
    if (!h || !variant) return ATSAT_DYN_E_INVALID;
    *variant = variant_available(h, h->variant) ? h->variant : ATSAT_DYN_STAGE_DIRECT;
    return ATSAT_DYN_OK;
}

int atsat_dyn_autotune(atsat_dyn_t h, int32_t reps, int32_t* chosen, double* ms) {
    ENTRY(h);
    if (!chosen || !ms || reps < 1) return fail(h, ATSAT_DYN_E_INVALID, "autotune: bad arguments");
    if (h->p.precision != ATSAT_DYN_MIXED)
        return fail(h, ATSAT_DYN_E_UNSUPPORTED, "autotune applies to the mixed-precision stage kernel");
    // stage 1 of a step: A -> B, the widest stage input (y_n, w's low word and the increments)
    StageParams sp{};
    sp.stage = 1;
    sp.c_in = 0.5 * h->p.dt;
    sp.wgt = 2.0;
    sp.sixth_dt = h->p.dt / 6.0;
    sp.c_in_f = (float)sp.c_in;
    sp.wgt_f = (float)sp.wgt;
    sp.sixth_dt_f = (float)sp.sixth_dt;
    const MixedIO io = make_mixed_io(h, h->dlA, h->dlB, nullptr);
    const int keep = h->variant;
    cudaEvent_t ev[2];
    CK(h, cudaEventCreate(&ev[0]));
    CK(h, cudaEventCreate(&ev[1]));
    int best = -1;
    auto time_stage = [&](double* out) -> int {
        for (int r = 0; r < 2 + reps; r++) {
            if (r == 2) CK(h, cudaEventRecord(ev[0], h->stream));
            CK(h, launch_stage(h, io, sp, MODE_STAGE));
            h->launches += launches_per_stage(h);
        }
        CK(h, cudaEventRecord(ev[1], h->stream));
        CK(h, cudaEventSynchronize(ev[1]));
        float t = 0.0f;
        CK(h, cudaEventElapsedTime(&t, ev[0], ev[1]));
        *out = t / reps;
        return ATSAT_DYN_OK;
    };
    int best_levels = h->march_levels;
    for (int v = 0; v < ATSAT_DYN_STAGE_NVARIANT; v++) {
        ms[v] = -1.0;
        if (!variant_available(h, v)) continue;
        h->variant = v;
        if (v == ATSAT_DYN_STAGE_MARCH) {
            // the march depth: whole columns, halves, thirds, quarters, and short runs
            const int n = h->kc.im - 2;
            std::vector<int> cand = {default_march_levels(h), n, (n + 1) / 2, (n + 2) / 3, (n + 3) / 4, 8, 4};
            for (int lv : cand) {
                if (lv < 1 || lv > n) continue;
                h->march_levels = lv;
                double t = 0.0;
                const int rc = time_stage(&t);
                if (rc) return rc;
                if (ms[v] < 0.0 || t < ms[v]) { ms[v] = t; best_levels = lv; }
            }
            h->march_levels = best_levels;
        } else {
            const int rc = time_stage(&ms[v]);
            if (rc) return rc;
        }
        if (best < 0 || ms[v] < ms[best]) best = v;
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    h->variant = best >= 0 ? best : keep;
    h->march_levels = best_levels;
    *chosen = h->variant;
    const int rc = finish(h, true);
    if (rc == ATSAT_DYN_OK && best >= 0) tune_cache_store(h, ms[best]);
    return rc;
}

// ---- standalone pressure-equation solves ----

static int poisson_ready(atsat_dyn* h) {
    if (h->poisson) return ATSAT_DYN_OK;
    std::string err;
    h->poisson = poisson_create(h->kc, h->geo, h->geo_h, h->stream, &err);
    if (!h->poisson) return fail(h, err.find("cudaMalloc") != std::string::npos ? ATSAT_DYN_E_NOMEM : ATSAT_DYN_E_UNSUPPORTED,
                                 "%s", err.c_str());
    return ATSAT_DYN_OK;
}

int atsat_dyn_poisson_project(atsat_dyn_t h, double* src) {
    ENTRY(h);
    if (!src) return fail(h, ATSAT_DYN_E_INVALID, "poisson_project: null source");
    int rc;
    if ((rc = poisson_ready(h))) return rc;
    const KConst& K = h->kc;
    const std::vector<double>& y = poisson_null_vector(h->poisson);
    const int NI = K.im - 2, NJ = K.jm - 2, n = K.km - 1;
    // the phi-mean of the source is its zero-mode part; remove its component along y
    double yf = 0.0, yy = 0.0;
    std::vector<double> mean((size_t)NI * NJ);
    for (int jj = 0; jj < NJ; jj++)
        for (int ii = 0; ii < NI; ii++) {
            const double* row = src + ((size_t)(ii + 1) * K.jm + (jj + 1)) * K.km;
            double a = 0.0;
            for (int k = 0; k < n; k++) a += row[k];
            mean[(size_t)jj * NI + ii] = a / n;
            const double yv = y[(size_t)jj * NI + ii];
            yf += yv * a / n;
            yy += yv * yv;
        }
    if (!(yy > 0.0)) return fail(h, ATSAT_DYN_E_INVALID, "poisson_project: degenerate null vector");
    const double alpha = yf / yy;
    for (int jj = 0; jj < NJ; jj++)
        for (int ii = 0; ii < NI; ii++) {
            double* row = src + ((size_t)(ii + 1) * K.jm + (jj + 1)) * K.km;
            const double d = alpha * y[(size_t)jj * NI + ii];
            for (int k = 0; k < K.km; k++) row[k] -= d;
        }
    return ATSAT_DYN_OK;
}

int atsat_dyn_poisson_solve(atsat_dyn_t h, int32_t method, const double* src, double* p, double tol,
                            int32_t max_iter, int32_t inner, double omega, atsat_dyn_poisson_stats* st) {
    ENTRY(h);
    if (!src || !p || method < 0 || method >= ATSAT_POISSON_NMETHOD || max_iter < 0 || !(omega > 0.0 && omega < 2.0))
        return fail(h, ATSAT_DYN_E_INVALID, "poisson_solve: bad arguments");
    if ((method == ATSAT_POISSON_REFINE_SOR) && inner < 1)
        return fail(h, ATSAT_DYN_E_INVALID, "poisson_solve: inner sweeps < 1");
    int rc;
    if ((rc = poisson_ready(h))) return rc;
    const KConst& K = h->kc;
    double* f = poisson_f(h->poisson);
    CK(h, cudaMemcpy2DAsync(f, (size_t)K.kp * 8, src, (size_t)K.km * 8, (size_t)K.km * 8, (size_t)K.im * K.jm,
                            cudaMemcpyHostToDevice, h->stream));
    cudaEvent_t ev[2];
    CK(h, cudaEventCreate(&ev[0]));
    CK(h, cudaEventCreate(&ev[1]));
    CK(h, cudaEventRecord(ev[0], h->stream));
    int iters = 0, inner_total = 0;
    double rel = 0.0;
    CK(h, poisson_run(h->poisson, method, tol, max_iter, inner, omega, &iters, &inner_total, &rel));
    CK(h, cudaEventRecord(ev[1], h->stream));
    CK(h, cudaEventSynchronize(ev[1]));
    float ms = 0.0f;
    CK(h, cudaEventElapsedTime(&ms, ev[0], ev[1]));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    CK(h, cudaMemcpy2DAsync(p, (size_t)K.km * 8, poisson_p(h->poisson), (size_t)K.kp * 8, (size_t)K.km * 8,
                            (size_t)K.im * K.jm, cudaMemcpyDeviceToHost, h->stream));
    if (st) {
        memset(st, 0, sizeof(*st));
        st->method = method;
        st->iterations = iters;
        st->inner = inner_total;
        st->converged = rel <= tol;
        st->rel_residual = rel;
        st->ms = ms;
        int spp = 0;
        double sms = 0.0;
        poisson_sweep_stats(h->poisson, &spp, &sms);
        st->sweeps_per_pass = spp;
        st->sweep_ms = sms;
    }
    return finish(h, true);
}

}  // extern "C"
