// Test infrastructure: drives the REFERENCE's own hot path (compiled from the reference sources
// where they lie, see oracle/build_ref.py) on injected state, to pin the CPU restatement in
// oracle/atsat_oracle.c. Nothing in the product links or runs this.
//
// How it reaches private members without editing the reference: cSaturnModel befriends every
// specialisation of ProcessDiag (planet/cSaturnModel.h:61, 83), so a full specialisation for a
// tag type of our own is a friend too.
//
// Usage: ref_harness <in.bin> <out.bin> <op> [nsteps] [iter0]
//   op = rhs       one RHSSat pass over the RK interior (RungeKutta_Sat_Turb.cpp:220-247) after
//                  computeBuoyancyRefLevel / computeMetricPressure, on the live fields
//        rk        cSaturnModel::RungeKuttaSat()
//        pressure  PressureSolver<cSaturnModel>::run()
//        density   cSaturnModel::computeMixtureDensity()
//        steps     nsteps iterations of the dycore sequence of cSaturnModel::Run
//                  (cSaturnModel.cpp:864-1111 restricted to the dycore): on even iterations
//                  computeMixtureDensity + pressure; then RungeKuttaSat; bcTheta, bcPhi, bcRadius;
//                  restoreVar(1.0). Iterations run iter0 .. iter0+nsteps-1 (iter0 defaults to 1).
//        damp      the p_dyn filter Run applies after the pressure call (cSaturnModel.cpp:894-897)
//        clamp     cSaturnModel::clampNegativeSpecies() (FileIO_Sat.cpp:716-772); writes its budget
//        driver    as steps, with damp after the pressure call, clamp after the boundary conditions and
//                  the turbulence closure after restoreVar (cSaturnModel.cpp:894-897, 1101, 1116)
//        turb      TurbulenceSat(m).run() (Turbulence.h:306-329); writes prod, vel_star and the constants
//        save      cSaturnModel::save_state(nsteps) into $ORACLE_RESTART_DIR (FileIO_Sat.cpp:578-613)
// Record format of both files: char name[48]; int64 count; double data[count].

#include "cSaturnModel.h"
#include "ProcessDiag.h"
#include "PressureSolverSat.h"
#include "BC_Sat.h"
#include "TurbulenceSat.h"
#include "Utils.h"
#include "ATPhys.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

struct OracleTag {};

template<>
class ProcessDiag<OracleTag> {
public:
    typedef std::map<std::string, std::vector<double> > Records;

    static bool read_records(const char* path, Records& out){
        FILE* f = fopen(path, "rb");
        if(!f) return false;
        for(;;){
            char name[48];
            int64_t n;
            if(fread(name, 1, 48, f) != 48) break;
            if(fread(&n, 8, 1, f) != 1){ fclose(f); return false; }
            std::vector<double> v((size_t)n);
            if(n > 0 && fread(v.data(), 8, (size_t)n, f) != (size_t)n){ fclose(f); return false; }
            name[47] = 0;
            out[std::string(name)] = v;
        }
        fclose(f);
        return true;
    }

    static void write_record(FILE* f, const std::string& name, const double* d, int64_t n){
        char buf[48];
        memset(buf, 0, 48);
        strncpy(buf, name.c_str(), 47);
        fwrite(buf, 1, 48, f);
        fwrite(&n, 8, 1, f);
        if(n) fwrite(d, 8, (size_t)n, f);
    }

    static std::map<std::string, Array*> field_table(cSaturnModel& m){
        std::map<std::string, Array*> t;
#define F_(x) t[#x] = &m.x;
        F_(u) F_(v) F_(w) F_(t) F_(h2o) F_(h2o_cloud) F_(h2o_ice) F_(h2s) F_(nh3) F_(nh3_cloud)
        F_(nh3_ice) F_(ch4) F_(ch4_cloud) F_(ch4_ice) F_(nh4sh) F_(tke) F_(dis)
        F_(un) F_(vn) F_(wn) F_(tn) F_(h2on) F_(h2o_cloudn) F_(h2o_icen) F_(h2sn) F_(nh3n)
        F_(nh3_cloudn) F_(nh3_icen) F_(ch4n) F_(ch4_cloudn) F_(ch4_icen) F_(nh4shn) F_(tken) F_(disn)
        F_(p_dyn) F_(p_stat) F_(p_metric) F_(rho_mix)
        F_(nue) F_(Q_precip) F_(Q_rad) F_(tke_source) F_(dis_source)
        F_(S_precip_h2o) F_(S_precip_h2o_cloud) F_(S_precip_h2o_ice)
        F_(S_precip_nh3) F_(S_precip_nh3_cloud) F_(S_precip_nh3_ice)
        F_(S_precip_ch4) F_(S_precip_ch4_cloud) F_(S_precip_ch4_ice)
        F_(massflux_h2s) F_(massflux_nh3) F_(massflux_nh4sh) F_(fluxlim_nh4sh) F_(thermalmassflux)
        F_(rhs_u) F_(rhs_v) F_(rhs_w) F_(rhs_t) F_(rhs_h2o) F_(rhs_h2o_cloud) F_(rhs_h2o_ice)
        F_(rhs_h2s) F_(rhs_nh3) F_(rhs_nh3_cloud) F_(rhs_nh3_ice) F_(rhs_ch4) F_(rhs_ch4_cloud)
        F_(rhs_ch4_ice) F_(rhs_nh4sh) F_(rhs_tke) F_(rhs_dis)
        F_(aux_u) F_(aux_v) F_(aux_w) F_(p_dynn)
#undef F_
        return t;
    }

    static void load_array(cSaturnModel& m, Array& a, const std::vector<double>& d){
        const int im = m.im, jm = m.jm, km = m.km;
        for(int i = 0; i < im; i++) for(int j = 0; j < jm; j++) for(int k = 0; k < km; k++)
            a.x[i][j][k] = d[((size_t)i * jm + j) * km + k];
    }

    static void dump_array(cSaturnModel& m, FILE* f, const std::string& name, Array& a){
        const int im = m.im, jm = m.jm, km = m.km;
        std::vector<double> d((size_t)im * jm * km);
        for(int i = 0; i < im; i++) for(int j = 0; j < jm; j++) for(int k = 0; k < km; k++)
            d[((size_t)i * jm + j) * km + k] = a.x[i][j][k];
        write_record(f, name, d.data(), (int64_t)d.size());
    }

    // The p_dyn filter of cSaturnModel::Run after the pressure call (cSaturnModel.cpp:894-897), with its
    // mode chosen as Run chooses it.
    static void damp_pdyn(cSaturnModel& m){
        const char* e = getenv("ATSAT_DAMP_PDYN");
        const int mode = e ? atoi(e) : (cSaturnModel::geo_balance() ? 3 : 1);
        if(mode == 1)      AtomUtils::damp_wiggles(m.p_dyn, nullptr, true, true, true);
        else if(mode == 2) AtomUtils::damp_wiggles(m.p_dyn, nullptr, true, false, false);
        else if(mode == 3) AtomUtils::damp_wiggles(m.p_dyn, nullptr, true, false, true);
    }

    // One RHSSat pass with the per-column geometry RungeKuttaSat builds
    // (RungeKutta_Sat_Turb.cpp:129-142, 223-245).
    static void rhs_pass(cSaturnModel& m){
        m.computeBuoyancyRefLevel();
        if(m.metric_split()) m.computeMetricPressure();
        const int im = m.im, jm = m.jm, km = m.km;
        std::vector<double> st(jm), ct(jm);
        const double s_min = m.sinthe_min();
        for(int j = 0; j < jm; j++){
            st[j] = sin(m.the.z[j]);
            if(st[j] < s_min) st[j] = s_min;
            ct[j] = cos(m.the.z[j]);
        }
        const int k_first = ATPhys::phi_first(ATPhys::phi_periodic<cSaturnModel>());
        #pragma omp parallel for collapse(2) schedule(static)
        for(int i = 1; i < im-1; i++){
            for(int j = 2; j < jm-2; j++){
                cSaturnModel::CellGeometry geo;
                geo.rm       = m.metricRadius(m.rad.z[i]);
                geo.rm2      = geo.rm * geo.rm;
                geo.exp_rm   = m.coord_stretching ? 1.0 / (geo.rm + 1.0) : 1.0;
                geo.exp_2_rm = geo.exp_rm * geo.exp_rm;
                geo.sinthe   = st[j];
                geo.sinthe2  = geo.sinthe * geo.sinthe;
                geo.costhe   = ct[j];
                geo.cotanthe             = geo.costhe / geo.sinthe;
                geo.inv_rm               = 1.0 / geo.rm;
                geo.inv_rm2              = 1.0 / geo.rm2;
                geo.inv_rmsinthe         = 1.0 / (geo.rm * geo.sinthe);
                geo.inv_rm2sinthe        = geo.inv_rm2 / geo.sinthe;
                geo.inv_rm2sinthe2       = geo.inv_rm2 / geo.sinthe2;
                geo.costhe_inv_rm2sinthe = geo.costhe * geo.inv_rm2sinthe;
                geo.inv_2dr   = 1.0 / (2.0 * m.dr);
                geo.inv_2dthe = 1.0 / (2.0 * m.dthe);
                geo.inv_2dphi = 1.0 / (2.0 * m.dphi);
                geo.inv_dr2   = 1.0 / (m.dr * m.dr);
                geo.inv_dthe2 = 1.0 / (m.dthe * m.dthe);
                geo.inv_dphi2 = 1.0 / (m.dphi * m.dphi);
                for(int k = k_first; k < km-1; k++) m.RHSSat(i, j, k, geo);
            }
        }
    }

    static int main(int argc, char** argv){
        if(argc < 4){ fprintf(stderr, "usage: ref_harness in.bin out.bin op [nsteps] [iter0]\n"); return 2; }
        // Run() sets this before its loop under the default GEO_BALANCE (cSaturnModel.cpp:612).
        setenv("ATSAT_PRESS_INCR", "1", 0);
        Records in;
        if(!read_records(argv[1], in)){ fprintf(stderr, "cannot read %s\n", argv[1]); return 2; }
        const std::string op = argv[3];
        const int nsteps = argc > 4 ? atoi(argv[4]) : 1;
        const int iter0 = argc > 5 ? atoi(argv[5]) : 1;

        cSaturnModel* mp = new cSaturnModel();
        cSaturnModel& m = *mp;
        m.resetArrays();
        m.ThermalPropertiesSat();
        m.turb_active = true;
        m.dt = 0.01;
        m.re = 100000.0;            // the committed configuration, cli/config_atsat.xml
        m.pr = 69.0;
        for(auto& kv : in){
            if(kv.first.compare(0, 6, "param:") == 0){
                const std::string p = kv.first.substr(6);
                const double x = kv.second.at(0);
                if(p == "re") m.re = x;
                else if(p == "pr") m.pr = x;
                else if(p == "dt") m.dt = x;
                else if(p == "turb_active") m.turb_active = (x != 0.0);
                else { fprintf(stderr, "unknown param %s\n", p.c_str()); return 2; }
            }
        }
        std::map<std::string, Array*> tab = field_table(m);
        for(auto& kv : in){
            auto it = tab.find(kv.first);
            if(it != tab.end()){
                if(kv.second.size() != (size_t)m.im * m.jm * m.km){ fprintf(stderr, "bad size %s\n", kv.first.c_str()); return 2; }
                load_array(m, *it->second, kv.second);
            }
        }
        if(in.count("cell_vbar0")){ m.cell_vbar0 = in["cell_vbar0"]; m.cell_ubar0 = in["cell_ubar0"]; }
        if(in.count("p_baro")) m.p_baro = in["p_baro"];

        if(op == "rhs") rhs_pass(m);
        else if(op == "rk") m.RungeKuttaSat();
        else if(op == "pressure") m.getPressureSolver().run();
        else if(op == "density") m.computeMixtureDensity();
        else if(op == "steps"){
            for(int it = iter0; it < iter0 + nsteps; it++){
                if(it % 2 == 0){
                    m.computeMixtureDensity();
                    m.getPressureSolver().run();
                }
                m.RungeKuttaSat();
                BC_Sat(m).bcTheta();
                BC_Sat(m).bcPhi();
                BC_Sat(m).bcRadius();
                m.restoreVar(1.0);
            }
        } else if(op == "damp"){
            AtomUtils::set_phi_seam_periodic(ATPhys::phi_periodic<cSaturnModel>());   // as Run() does
            damp_pdyn(m);
        } else if(op == "clamp"){
            m.clampNegativeSpecies();
        } else if(op == "turb"){
            TurbulenceSat(m).run();
        } else if(op == "save"){
            // cSaturnModel::save_state (FileIO_Sat.cpp:578-613) into ORACLE_RESTART_DIR, iteration = nsteps
            const char* d = getenv("ORACLE_RESTART_DIR");
            m.output_path = d ? d : ".";
            m.save_state(nsteps);
        } else if(op == "driver"){
            // the dycore sequence with the driver's glue around it: the p_dyn filter after the pressure
            // call (cSaturnModel.cpp:894-897) and the species floor after the boundary conditions (:1101)
            AtomUtils::set_phi_seam_periodic(ATPhys::phi_periodic<cSaturnModel>());
            for(int it = iter0; it < iter0 + nsteps; it++){
                if(it % 2 == 0){
                    m.computeMixtureDensity();
                    m.getPressureSolver().run();
                    damp_pdyn(m);
                }
                m.RungeKuttaSat();
                BC_Sat(m).bcTheta();
                BC_Sat(m).bcPhi();
                BC_Sat(m).bcRadius();
                m.clampNegativeSpecies();
                m.restoreVar(1.0);
                if(m.turb_active) TurbulenceSat(m).run();
            }
        } else { fprintf(stderr, "unknown op %s\n", op.c_str()); return 2; }

        FILE* f = fopen(argv[2], "wb");
        if(!f){ fprintf(stderr, "cannot write %s\n", argv[2]); return 2; }
        for(auto& kv : tab) dump_array(m, f, kv.first, *kv.second);
        write_record(f, "buoy_ref_level", m.buoy_ref_level.data(), (int64_t)m.buoy_ref_level.size());
        const double consts[] = { m.re, m.pr, m.sc_h2o, m.sc_nh3, m.sc_h2s, m.sc_ch4, m.sc_nh4sh,
                                  m.u_0, m.t_ref, m.L_atm, m.g, m.omega, m.Coriolis, m.centrifugal,
                                  m.buoyancy, m.chemical_reaction, m.cp_mix, m.r_mix, m.R_mix, m.dt,
                                  m.dr, m.dthe, m.dphi };
        const char* cnames[] = { "re", "pr", "sc_h2o", "sc_nh3", "sc_h2s", "sc_ch4", "sc_nh4sh",
                                 "u_0", "t_ref", "L_atm", "g", "omega", "Coriolis", "centrifugal",
                                 "buoyancy", "chemical_reaction", "cp_mix", "r_mix", "R_mix", "dt",
                                 "dr", "dthe", "dphi" };
        for(size_t c = 0; c < sizeof(consts) / sizeof(consts[0]); c++)
            write_record(f, std::string("const:") + cnames[c], &consts[c], 1);
        if(!m.clamp_added.empty()){
            const size_t nf = m.clamp_added.size();
            std::vector<double> cells(nf), cells_bnd(nf);
            for(size_t q = 0; q < nf; q++){ cells[q] = (double)m.clamp_cells[q]; cells_bnd[q] = (double)m.clamp_cells_bnd[q]; }
            write_record(f, "clamp_added", m.clamp_added.data(), (int64_t)nf);
            write_record(f, "clamp_cells", cells.data(), (int64_t)nf);
            write_record(f, "clamp_added_bnd", m.clamp_added_bnd.data(), (int64_t)nf);
            write_record(f, "clamp_cells_bnd", cells_bnd.data(), (int64_t)nf);
        }
        {
            std::vector<double> vs((size_t)m.jm * m.km);
            for(int j = 0; j < m.jm; j++) for(int k = 0; k < m.km; k++) vs[(size_t)j * m.km + k] = m.vel_star.y[j][k];
            write_record(f, "vel_star", vs.data(), (int64_t)vs.size());
            dump_array(m, f, "prod", m.prod);
            const double tc[] = { m.ep_h2o, m.ep_nh3, m.ep_ch4, m.lv_h2o, m.lv_nh3, m.lv_ch4, m.ls_h2o, m.ls_nh3,
                                  m.ls_ch4, m.t_0_h2o, m.t_0_nh3, m.t_0_ch4, m.abl_height };
            write_record(f, "turb_consts", tc, (int64_t)(sizeof(tc) / sizeof(tc[0])));
        }
        write_record(f, "rad_z", m.rad.z, m.im);
        write_record(f, "the_z", m.the.z, m.jm);
        fclose(f);
        return 0;
    }
};

int main(int argc, char** argv){ return ProcessDiag<OracleTag>::main(argc, argv); }
