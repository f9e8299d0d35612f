// The drop-in adapter between MolTwister's `moldyn run` / `moldyn optimizeenergy` and libmtgpu.so:
// builds the two descriptors of include/mtgpu.h from the reference's own objects.
//
//   atoms, types (first-appearance order), molecule indices, the 1000-point tables
//                              : CMDFFMatrices, the reference's prepareFFMatrices
//                                (ForceFields/MDFFMatrices.cpp:181-536)
//   term kinds and parameters  : the MDFF lists (getFFType, getArguments), MDFF/**
//   bonds, angles, dihedrals   : CMolTwisterStateTools::getAll{MDBonds,MDAngles,MDDihedrals}InSystem
//                                (MolTwisterStateTools.cpp:544-1209)
//   run settings               : SMolDynConfigStruct (Config/MolDynConfigStruct.h:24-65)
//
// and runs a simulation through the C ABI (run()).  It compiles against the reference headers
// and is built with the reference's CPU MD sources by oracle/ref/Makefile into the test harness,
// where `mtref desc` dumps the descriptors it produces for comparison with the Python binding's
// (tests/test_adapter.py); the MolTwister host build would compile the same file.
#include "adapter.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sstream>

#include "Cmd/MolTwisterCmdMolDyn/ForceFields/MDFFMatrices.h"
#include "Cmd/Tools/MolTwisterStateTools.h"

namespace mtgpu_adapter {
namespace {

// The numbers of a term's getArguments() string ("name:value name:value ..."), in order: the
// parse order of the term's command, which is the parameter order of the mtg_term kinds.
std::vector<double> argument_values(const std::string& args) {
    std::vector<double> v;
    std::istringstream is(args);
    std::string tok;
    while(is >> tok) {
        const size_t c = tok.find(':');
        if(c != std::string::npos) v.push_back(strtod(tok.c_str() + c + 1, nullptr));
    }
    return v;
}

int nb_kind(const std::string& t) {
    if(t == "LJ") return MTG_NB_LJ;
    if(t == "LJ1208") return MTG_NB_LJ1208;
    if(t == "Buck") return MTG_NB_BUCK;
    if(t == "LJBuck") return MTG_NB_LJBUCK;
    return -1;
}
int bond_kind(const std::string& t) {
    if(t == "Harm") return MTG_BOND_HARM;
    if(t == "Morse") return MTG_BOND_MORSE;
    if(t == "LJC") return MTG_BOND_LJC;
    return -1;
}
int angle_kind(const std::string& t) {
    if(t == "Harm") return MTG_ANGLE_HARM;
    if(t == "Class2") return MTG_ANGLE_CLASS2;
    return -1;
}
int dih_kind(const std::string& t) {
    if(t == "Harm") return MTG_DIH_HARM;
    if(t == "Fourier4t") return MTG_DIH_FOURIER4T;
    return -1;
}

mtg_term make_term(int kind, const std::vector<double>& v) {
    mtg_term t{};
    t.kind = kind;
    for(size_t k = 0; k < v.size() && k < 4; k++) t.p[k] = v[k];
    if(kind == MTG_ANGLE_HARM) t.p[2] = 0.017453292519943295;   // CMDFFAngle_Harm::toRad_
    return t;
}

void copy_table(const mtdevice_vector<CMDFFMatrices::CPoint>& src, std::vector<float>& dst) {
    dst.clear();
    for(const auto& p : src) {
        dst.push_back(p.x_);
        dst.push_back(p.f_);
        dst.push_back(p.e_);
    }
}

}  // namespace

bool build(CMolTwisterState* st, const SMolDynConfigStruct& cfg, Descriptors& d, std::string& err) {
    d = Descriptors{};
    CMDFFMatrices M(st, stdout, (float)cfg.cutoffRadius_, (float)cfg.neighListShell_);
    const int N = M.getNumAtoms(), T = M.getNumAtomTypes();
    if(N <= 0) {
        err = "no atoms";
        return false;
    }
    // ---- atoms ----
    d.r.resize(3 * (size_t)N);
    d.mass.resize(N);
    d.charge.resize(N);
    d.type.resize(N);
    d.mol.resize(N);
    d.mobile.resize(N);
    d.type_names.assign(T, std::string());
    const int frame = st->currentFrame_;
    for(int k = 0; k < N; k++) {
        const CAtom* a = st->atoms_[k].get();
        const C3DVector r = a->r_[frame < (int)a->r_.size() ? frame : 0];
        d.r[3 * k] = r.x_;
        d.r[3 * k + 1] = r.y_;
        d.r[3 * k + 2] = r.z_;
        d.mass[k] = a->m_;
        d.charge[k] = a->Q_;
        d.type[k] = M.devAtomList_[k].typeIndex_;
        d.mol[k] = M.devAtomList_[k].molIndex_;
        d.mobile[k] = a->isMobile_ ? 1 : 0;
        if(d.type_names[d.type[k]].empty()) d.type_names[d.type[k]] = a->getID();
    }
    // ---- non-bonded terms per (row, col) type pair, in the MDFF list's order ----
    d.nb_count.assign((size_t)T * T, 0);
    d.nb_terms.assign((size_t)T * T * MTG_MAX_FF_PER_PAIR, mtg_term{});
    for(int row = 0; row < T; row++)
        for(int col = 0; col < T; col++) {
            std::shared_ptr<std::vector<int>> idx = st->mdFFNonBondedList_.indexFromNames(d.type_names[row], d.type_names[col]);
            int n = 0;
            for(int i : *idx) {
                if(n >= MTG_MAX_FF_PER_PAIR) break;
                CMDFFNonBonded* term = st->mdFFNonBondedList_.get(i);
                const int kind = nb_kind(term->getFFType());
                if(kind < 0) {
                    err = "non-bonded term kind " + term->getFFType() + " has no counterpart in libmtgpu";
                    return false;
                }
                std::vector<double> v = argument_values(term->getArguments(false));
                if(kind == MTG_NB_LJ || kind == MTG_NB_LJ1208) v.resize(3);   // epsilon, sigma, alpha; rc = 0
                d.nb_terms[((size_t)row * T + col) * MTG_MAX_FF_PER_PAIR + n] = make_term(kind, v);
                n++;
            }
            d.nb_count[(size_t)row * T + col] = n;
        }
    // the reference's tables, point index outermost (MDFFMatrices.cpp:538-541), reordered to the
    // library's [((row T + col) 5 + ff) 1000 + point] layout
    {
        const size_t P = MTG_NPTS, F = MTG_MAX_FF_PER_PAIR;
        d.nb_tables.assign((size_t)T * T * F * P * 3, 0.0f);
        for(size_t j = 0; j < P; j++)
            for(size_t ff = 0; ff < F; ff++)
                for(int row = 0; row < T; row++)
                    for(int col = 0; col < T; col++) {
                        const size_t src = (size_t)T * ((size_t)T * (F * j + ff) + row) + col;
                        if(src >= M.devNonBondFFMatrix_.size()) continue;
                        const auto& pt = M.devNonBondFFMatrix_[src];
                        const size_t dst = ((((size_t)row * T + col) * F + ff) * P + j) * 3;
                        d.nb_tables[dst] = pt.x_;
                        d.nb_tables[dst + 1] = pt.f_;
                        d.nb_tables[dst + 2] = pt.e_;
                    }
    }
    // ---- bonded term types, their tables and the topology ----
    for(int t = 0; t < st->mdFFBondList_.size(); t++) {
        CMDFFBond* b = st->mdFFBondList_.get(t);
        const int kind = bond_kind(b->getFFType());
        if(kind < 0) { err = "bond kind " + b->getFFType() + " has no counterpart"; return false; }
        d.bond_terms.push_back(make_term(kind, argument_values(b->getArguments(false))));
    }
    for(int t = 0; t < st->mdFFAngleList_.size(); t++) {
        CMDFFAngle* a = st->mdFFAngleList_.get(t);
        const int kind = angle_kind(a->getFFType());
        if(kind < 0) { err = "angle kind " + a->getFFType() + " has no counterpart"; return false; }
        d.angle_terms.push_back(make_term(kind, argument_values(a->getArguments(false))));
    }
    for(int t = 0; t < st->mdFFDihList_.size(); t++) {
        CMDFFDih* h = st->mdFFDihList_.get(t);
        const int kind = dih_kind(h->getFFType());
        if(kind < 0) { err = "dihedral kind " + h->getFFType() + " has no counterpart"; return false; }
        d.dih_terms.push_back(make_term(kind, argument_values(h->getArguments(false))));
    }
    copy_table(M.devBondFFList_, d.bond_tables);
    copy_table(M.devAngleFFList_, d.angle_tables);
    copy_table(M.devDihedralFFList_, d.dih_tables);
    {
        std::vector<int> b1, b2, bt, a1, a2, a3, at, d1, d2, d3, d4, dt;
        CMolTwisterStateTools tools(st, stdout);
        tools.getAllMDBondsInSystem(b1, b2, bt, true);
        tools.getAllMDAnglesInSystem(a1, a2, a3, at, true);
        tools.getAllMDDihedralsInSystem(d1, d2, d3, d4, dt, true);
        for(size_t j = 0; j < b1.size(); j++) d.bonds.insert(d.bonds.end(), {b1[j], b2[j], bt[j]});
        for(size_t j = 0; j < a1.size(); j++) d.angles.insert(d.angles.end(), {a1[j], a2[j], a3[j], at[j]});
        for(size_t j = 0; j < d1.size(); j++) d.dihedrals.insert(d.dihedrals.end(), {d1[j], d2[j], d3[j], d4[j], dt[j]});
    }
    // ---- the descriptors ----
    mtg_system_desc& s = d.sys;
    s.n_atoms = N;
    s.n_types = T;
    s.r = d.r.data();
    s.p = nullptr;
    s.mass = d.mass.data();
    s.charge = d.charge.data();
    s.type = d.type.data();
    s.mol = d.mol.data();
    s.mobile = d.mobile.data();
    const C3DRect pbc = st->view3D_->calcPBC();
    s.box[0] = pbc.getWidthX();
    s.box[1] = pbc.getWidthY();
    s.box[2] = pbc.getWidthZ();
    s.nb_count = d.nb_count.data();
    s.nb_terms = d.nb_terms.data();
    s.nb_tables = d.nb_tables.data();
    s.n_bond_types = (int32_t)d.bond_terms.size();
    s.bond_terms = d.bond_terms.empty() ? nullptr : d.bond_terms.data();
    s.bond_tables = d.bond_tables.empty() ? nullptr : d.bond_tables.data();
    s.n_angle_types = (int32_t)d.angle_terms.size();
    s.angle_terms = d.angle_terms.empty() ? nullptr : d.angle_terms.data();
    s.angle_tables = d.angle_tables.empty() ? nullptr : d.angle_tables.data();
    s.n_dih_types = (int32_t)d.dih_terms.size();
    s.dih_terms = d.dih_terms.empty() ? nullptr : d.dih_terms.data();
    s.dih_tables = d.dih_tables.empty() ? nullptr : d.dih_tables.data();
    s.n_bonds = (int32_t)(d.bonds.size() / 3);
    s.bonds = d.bonds.empty() ? nullptr : d.bonds.data();
    s.n_angles = (int32_t)(d.angles.size() / 4);
    s.angles = d.angles.empty() ? nullptr : d.angles.data();
    s.n_dihedrals = (int32_t)(d.dihedrals.size() / 5);
    s.dihedrals = d.dihedrals.empty() ? nullptr : d.dihedrals.data();

    mtg_config_desc& c = d.cfg;
    c = mtg_config_desc{};
    c.ensemble = cfg.ensemble_ == SMolDynConfigStruct::ensembleNVT ? MTG_NVT
               : cfg.ensemble_ == SMolDynConfigStruct::ensembleNPT ? MTG_NPT : MTG_NVE;
    c.temperature_nh_len = cfg.temperatureNHChainLength_;
    c.temperature_respa = cfg.temperatureRESPASteps_;
    c.pressure_nh_len = cfg.pressureNHChainLength_;
    c.pressure_respa = cfg.pressureRESPASteps_;
    c.precision = MTG_PREC_REFERENCE;
    c.coulomb = MTG_COULOMB_ALLPAIRS;
    c.clip_forces = 1;
    c.timestep = cfg.timeStep_;
    c.temperature = cfg.temperature_;
    c.temperature_relax = cfg.temperatureRelaxationTime_;
    c.pressure = cfg.pressure_;
    c.pressure_relax = cfg.pressureRelaxationTime_;
    c.cutoff_radius = cfg.cutoffRadius_;
    c.neigh_shell = cfg.neighListShell_;
    c.cutoff_force = cfg.cutoffForce_;
    c.scale12 = cfg.scale12Interactions_;
    c.scale13 = cfg.scale13Interactions_;
    c.scale14 = cfg.scale14Interactions_;
    c.scale1N = cfg.scaleAbove14BondedInteractions_;
    c.coulomb_cutoff = cfg.cutoffRadius_;
    c.list_skin = 1.0;
    c.opt_learning_rate = cfg.gradientDescentLearningRate_;
    c.opt_accuracy = cfg.gradientDescentAccuracy_;
    c.opt_max_steps = cfg.gradientDescentMaxSteps_;
    c.device = 0;
    c.lj_shift = 0;
    c.initial_max_neighbours = 0;
    return true;
}

namespace {
struct InfoOut {
    FILE* out;
};
int print_info(const mtg_output* o, void* user) {
    // the columns of CMDLoop's info line (MDLoop.cpp:388-403), in the reference's units
    InfoOut* w = static_cast<InfoOut*>(user);
    fprintf(w->out, "\t%-15lld%-15.4f%-15.6f%-15.6f%-15.6f%-15.6f\r\n", (long long)o->step, o->T * 120.272,
            o->P * 16388.2461, o->V, o->U, o->K);
    return 0;
}
}  // namespace

std::string run(const SMolDynConfigStruct& cfg, FILE* out, CMolTwisterState* st, uint32_t seed) {
    Descriptors d;
    std::string err;
    if(!build(st, cfg, d, err)) return "Error: " + err;
    mtg_ctx* ctx = nullptr;
    if(mtg_create(&d.sys, &d.cfg, &ctx) != MTG_OK) return std::string("Error: ") + mtg_last_error(nullptr);
    std::string result;
    if(mtg_init_state(ctx, seed, MTG_INIT_REFERENCE) != MTG_OK) result = std::string("Error: ") + mtg_last_error(ctx);
    InfoOut w{out};
    if(result.empty() && mtg_run(ctx, cfg.numberOfTimeSteps_, cfg.outputStride_, print_info, &w) != MTG_OK)
        result = std::string("Error: ") + mtg_last_error(ctx);
    mtg_destroy(ctx);
    return result;
}

}  // namespace mtgpu_adapter
