// Oracle harness around MolTwister's own CPU molecular-dynamics path.
//
// TEST INFRASTRUCTURE ONLY.  This program is compiled (by oracle/ref/Makefile) from the unmodified
// reference sources plus this driver and a non-graphics C3DView stub; it never links into the
// product library, and nothing in the product calls it.  It is the parity anchor: the golden
// fixtures under tests/golden/ are its outputs.
//
// It builds a CMolTwisterState through the reference's public API (addAtom, Q_/m_/isMobile_, the
// MDFF list registries with the same parsing the `add md*` commands use:
// Cmd/MolTwisterCmdAdd/CmdMDNonBonded.cpp:72-114, CmdMDBond.cpp:81-152, CmdMDAngle.cpp,
// CmdMDDihedral.cpp), sets the user-defined periodic box, and then drives:
//   static : CMDFFMatrices (ForceFields/MDFFMatrices.cpp:117-179) -> tables, bonded lists, cell list,
//            neighbour list; CVelVerlet::calcParticleForces (Integrators/VelVerlet.cpp:152-158) -> F, Fpi, U
//   run    : CSimulationBox + the step sequence of CMDLoop::runSimulation (MDLoop/MDLoop.cpp:107-141)
//            with momenta and Nose-Hoover variables injected (they come from rand() otherwise,
//            SimulationBox.cpp:98-133, NHChain.cpp:126-143)
//   time   : the same step loop, wall-clock timed, for the CPU baseline.
//
// Input: a text system file (format written by moltwister_gb300/sysfile.py).  Output: "MTB1" named
// arrays (reader in oracle/mtb.py).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <string>
#include <vector>
#include <map>
#include <sstream>
#include <fstream>
#include <chrono>
#include <memory>

#include "MolTwisterState.h"
#include "Cmd/MolTwisterCmdMolDyn/ForceFields/MDFFMatrices.h"
#include "Cmd/MolTwisterCmdMolDyn/Integrators/VelVerlet.h"
#include "Cmd/MolTwisterCmdMolDyn/SimulationBox/SimulationBox.h"
#include "Cmd/MolTwisterCmdMolDyn/MDLoop/MDLoop.h"
#include "Cmd/MolTwisterCmdMolDyn/MDLoop/Printf.h"
#include "Cmd/MolTwisterCmdMolDyn/Config/MolDynConfig.h"
#include "Cmd/Tools/MolTwisterStateTools.h"
#include "Utilities/DCDFile.h"
#include "Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.h"
#include "adapter.h"
#include <functional>
#include <tuple>

namespace {

// ------------------------------------------------------------------------------------------------
// MTB1 writer: magic, then records {u32 namelen, name, u8 dtype, u32 ndim, u64 dims[], raw data}.
// ------------------------------------------------------------------------------------------------
class MtbWriter {
public:
    explicit MtbWriter(const std::string& path) {
        f_ = fopen(path.c_str(), "wb");
        if(!f_) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
        fwrite("MTB1", 1, 4, f_);
    }
    ~MtbWriter() { if(f_) fclose(f_); }
    template<class T> void put(const std::string& name, char dt, const std::vector<uint64_t>& dims, const T* data) {
        uint32_t n = (uint32_t)name.size();
        fwrite(&n, 4, 1, f_); fwrite(name.data(), 1, n, f_);
        uint8_t d = (uint8_t)dt; fwrite(&d, 1, 1, f_);
        uint32_t nd = (uint32_t)dims.size(); fwrite(&nd, 4, 1, f_);
        uint64_t cnt = 1;
        for(uint64_t x : dims) { fwrite(&x, 8, 1, f_); cnt *= x; }
        if(cnt) fwrite(data, sizeof(T), cnt, f_);
    }
    void d(const std::string& n, const std::vector<double>& v, std::vector<uint64_t> dims = {}) { if(dims.empty()) dims = {v.size()}; put(n, 'd', dims, v.data()); }
    void f(const std::string& n, const std::vector<float>& v, std::vector<uint64_t> dims = {}) { if(dims.empty()) dims = {v.size()}; put(n, 'f', dims, v.data()); }
    void i(const std::string& n, const std::vector<int32_t>& v, std::vector<uint64_t> dims = {}) { if(dims.empty()) dims = {v.size()}; put(n, 'i', dims, v.data()); }
private:
    FILE* f_ = nullptr;
};

// ------------------------------------------------------------------------------------------------
// System file
// ------------------------------------------------------------------------------------------------
struct AtomIn { std::string id; double x, y, z, q, m; int mobile; };
struct SysIn {
    double L[3] = {0, 0, 0};
    std::vector<AtomIn> atoms;
    std::vector<std::vector<std::string>> nonbonded, bonds, angles, dihedrals;
    std::map<std::string, std::string> cfg;
    std::vector<double> p;                 // injected momenta (3N) or empty
    std::vector<double> nhT_eta, nhT_peta, nhP_eta, nhP_peta;
    bool has_peps = false; double p_eps = 0.0;
};

std::vector<std::string> words(const std::string& line) {
    std::istringstream is(line); std::vector<std::string> w; std::string s;
    while(is >> s) w.push_back(s);
    return w;
}

SysIn readSys(const std::string& path) {
    std::ifstream in(path);
    if(!in) { fprintf(stderr, "cannot read %s\n", path.c_str()); exit(2); }
    SysIn s; std::string line;
    while(std::getline(in, line)) {
        auto w = words(line);
        if(w.empty() || w[0][0] == '#') continue;
        const std::string& k = w[0];
        if(k == "box") { for(int a = 0; a < 3; a++) s.L[a] = strtod(w[1 + a].c_str(), nullptr); }
        else if(k == "atom") {
            AtomIn a; a.id = w[1];
            a.x = strtod(w[2].c_str(), nullptr); a.y = strtod(w[3].c_str(), nullptr); a.z = strtod(w[4].c_str(), nullptr);
            a.q = strtod(w[5].c_str(), nullptr); a.m = strtod(w[6].c_str(), nullptr); a.mobile = atoi(w[7].c_str());
            s.atoms.push_back(a);
        }
        else if(k == "nonbonded") s.nonbonded.emplace_back(w.begin() + 1, w.end());
        else if(k == "bond") s.bonds.emplace_back(w.begin() + 1, w.end());
        else if(k == "angle") s.angles.emplace_back(w.begin() + 1, w.end());
        else if(k == "dihedral") s.dihedrals.emplace_back(w.begin() + 1, w.end());
        else if(k == "cfg") s.cfg[w[1]] = w[2];
        else if(k == "mom") { for(int a = 0; a < 3; a++) s.p.push_back(strtod(w[1 + a].c_str(), nullptr)); }
        else if(k == "nhT_eta") { for(size_t j = 1; j < w.size(); j++) s.nhT_eta.push_back(strtod(w[j].c_str(), nullptr)); }
        else if(k == "nhT_peta") { for(size_t j = 1; j < w.size(); j++) s.nhT_peta.push_back(strtod(w[j].c_str(), nullptr)); }
        else if(k == "nhP_eta") { for(size_t j = 1; j < w.size(); j++) s.nhP_eta.push_back(strtod(w[j].c_str(), nullptr)); }
        else if(k == "nhP_peta") { for(size_t j = 1; j < w.size(); j++) s.nhP_peta.push_back(strtod(w[j].c_str(), nullptr)); }
        else if(k == "p_eps") { s.has_peps = true; s.p_eps = strtod(w[1].c_str(), nullptr); }
        else { fprintf(stderr, "unknown key %s\n", k.c_str()); exit(2); }
    }
    return s;
}

// Detection criterion parsing, as in CmdMDBond.cpp:92-121 / CmdMDAngle.cpp (default all_r_less_than 1.75).
template<class Crit>
size_t parseCrit(const std::vector<std::string>& a, size_t arg, Crit& crit, double& r0, bool allow14) {
    const std::string t = arg < a.size() ? a[arg] : std::string();
    if(t == "all_r_less_than") { crit = (Crit)0; r0 = atof(a[arg + 1].c_str()); return arg + 2; }
    if(t == "mol_r_less_than") { crit = (Crit)1; r0 = atof(a[arg + 1].c_str()); return arg + 2; }
    if(t == "only_visible_bonds") { crit = (Crit)2; r0 = 0.0; return arg + 1; }
    if(allow14 && t == "only_14_bonds") { crit = (Crit)3; r0 = 0.0; return arg + 1; }
    crit = (Crit)0; r0 = 1.75; return arg;
}

void buildState(const SysIn& s, CMolTwisterState& st) {
    st.view3D_ = new C3DView(0, nullptr);
    CSerializer unused;
    st.view3D_->serialize(unused, false, &st.atoms_, &st.glObjects_, &st.currentFrame_, &st.defaultAtProp_);
    st.view3D_->setUserPBC(C3DRect(C3DVector(-s.L[0] / 2.0, -s.L[1] / 2.0, -s.L[2] / 2.0),
                                   C3DVector(s.L[0] / 2.0, s.L[1] / 2.0, s.L[2] / 2.0)));
    st.view3D_->enableUserPBC(true);
    for(const AtomIn& a : s.atoms) {
        int idx = st.addAtom(a.x, a.y, a.z, a.id);
        st.atoms_[idx]->Q_ = a.q;
        st.atoms_[idx]->m_ = a.m;
        st.atoms_[idx]->isMobile_ = (a.mobile != 0);
    }
    for(const auto& a : s.nonbonded) {
        std::shared_ptr<CMDFFNonBonded> e;
        for(int i = 0; i < st.mdFFNonBondedList_.getNumRegisteredFFTypes(); i++)
            if(a[2] == st.mdFFNonBondedList_.getRegisteredFFType(i)->getFFType()) { e = st.mdFFNonBondedList_.getRegisteredFFType(i)->createCopy(); break; }
        if(!e) { fprintf(stderr, "unknown nonbonded type %s\n", a[2].c_str()); exit(3); }
        e->setAtomsToBond(a[0], a[1]);
        if(!e->parse(std::vector<std::string>(a.begin() + 3, a.end()))) { fprintf(stderr, "parse error\n"); exit(3); }
        st.mdFFNonBondedList_.add(*e);
    }
    for(const auto& a : s.bonds) {
        std::shared_ptr<CMDFFBond> e;
        for(int i = 0; i < st.mdFFBondList_.getNumRegisteredFFTypes(); i++)
            if(a[2] == st.mdFFBondList_.getRegisteredFFType(i)->getFFType()) { e = st.mdFFBondList_.getRegisteredFFType(i)->createCopy(); break; }
        if(!e) { fprintf(stderr, "unknown bond type %s\n", a[2].c_str()); exit(3); }
        CMDFFBond::EDetCrit crit; double r0;
        size_t arg = parseCrit(a, 3, crit, r0, true);
        e->setAtomsToBond(a[0], a[1]);
        e->setBondDetectionCriteria(crit, r0);
        e->parse(std::vector<std::string>(a.begin() + arg, a.end()));
        st.mdFFBondList_.add(*e);
    }
    for(const auto& a : s.angles) {
        std::shared_ptr<CMDFFAngle> e;
        for(int i = 0; i < st.mdFFAngleList_.getNumRegisteredFFTypes(); i++)
            if(a[3] == st.mdFFAngleList_.getRegisteredFFType(i)->getFFType()) { e = st.mdFFAngleList_.getRegisteredFFType(i)->createCopy(); break; }
        if(!e) { fprintf(stderr, "unknown angle type %s\n", a[3].c_str()); exit(3); }
        CMDFFAngle::EDetCrit crit; double r0;
        size_t arg = parseCrit(a, 4, crit, r0, false);
        e->setAtomsToBond(a[0], a[1], a[2]);
        e->setBondDetectionCriteria(crit, r0);
        e->parse(std::vector<std::string>(a.begin() + arg, a.end()));
        st.mdFFAngleList_.add(*e);
    }
    for(const auto& a : s.dihedrals) {
        std::shared_ptr<CMDFFDih> e;
        for(int i = 0; i < st.mdFFDihList_.getNumRegisteredFFTypes(); i++)
            if(a[4] == st.mdFFDihList_.getRegisteredFFType(i)->getFFType()) { e = st.mdFFDihList_.getRegisteredFFType(i)->createCopy(); break; }
        if(!e) { fprintf(stderr, "unknown dihedral type %s\n", a[4].c_str()); exit(3); }
        CMDFFDih::EDetCrit crit; double r0;
        size_t arg = parseCrit(a, 5, crit, r0, false);
        e->setAtomsToBond(a[0], a[1], a[2], a[3]);
        e->setBondDetectionCriteria(crit, r0);
        e->parse(std::vector<std::string>(a.begin() + arg, a.end()));
        st.mdFFDihList_.add(*e);
    }
}

SMolDynConfigStruct makeCfg(const SysIn& s) {
    CMolDynConfig c;   // resetToDefaults(): Config/MolDynConfig.cpp:289-328
    for(const auto& kv : s.cfg) {
        std::string r = c.set(kv.first, kv.second);
        (void)r;
    }
    return c.cfg_;
}

std::vector<CParticle3D> particlesFromState(CMolTwisterState& st) {
    std::vector<CParticle3D> P(st.atoms_.size());
    for(size_t i = 0; i < P.size(); i++) { P[i].m_ = st.atoms_[i]->m_; P[i].r_ = st.atoms_[i]->r_[0]; }
    return P;
}

void dumpForces(MtbWriter& w, const std::string& pre, const std::vector<CMDFFMatrices::CForces>& F) {
    size_t N = F.size();
    std::vector<double> f(3 * N), fpi(3 * N); std::vector<float> u(N);
    for(size_t k = 0; k < N; k++) {
        f[3 * k] = F[k].F_.x_; f[3 * k + 1] = F[k].F_.y_; f[3 * k + 2] = F[k].F_.z_;
        fpi[3 * k] = F[k].Fpi_.x_; fpi[3 * k + 1] = F[k].Fpi_.y_; fpi[3 * k + 2] = F[k].Fpi_.z_;
        u[k] = F[k].U_;
    }
    w.d(pre + "F", f, {N, 3}); w.d(pre + "Fpi", fpi, {N, 3}); w.f(pre + "U", u);
}

// ------------------------------------------------------------------------------------------------
// static: tables, bonded lists, cell list, neighbour list, forces at the input positions
// ------------------------------------------------------------------------------------------------
int cmdStatic(const SysIn& s, const std::string& out) {
    CMolTwisterState st; buildState(s, st);
    SMolDynConfigStruct cfg = makeCfg(s);
    MtbWriter w(out);
    CMDFFMatrices M(&st, stdout, (float)cfg.cutoffRadius_, (float)cfg.neighListShell_);
    const int N = M.getNumAtoms(), T = M.getNumAtomTypes();

    std::vector<float> tab; std::vector<int32_t> cnt;
    for(const auto& p : M.devNonBondFFMatrix_) { tab.push_back(p.x_); tab.push_back(p.f_); tab.push_back(p.e_); }
    for(size_t c : M.devNonBondFFMatrixFFCount_) cnt.push_back((int32_t)c);
    w.f("nb_table", tab, {(uint64_t)tab.size() / 3, 3}); w.i("nb_count", cnt);
    auto dumpBondedTab = [&](const char* n, const mtdevice_vector<CMDFFMatrices::CPoint>& v) {
        std::vector<float> t; for(const auto& p : v) { t.push_back(p.x_); t.push_back(p.f_); t.push_back(p.e_); }
        w.f(n, t, {(uint64_t)t.size() / 3, 3});
    };
    dumpBondedTab("bond_table", M.devBondFFList_);
    dumpBondedTab("angle_table", M.devAngleFFList_);
    dumpBondedTab("dih_table", M.devDihedralFFList_);

    std::vector<int32_t> type(N), mol(N);
    for(int k = 0; k < N; k++) { type[k] = M.devAtomList_[k].typeIndex_; mol[k] = M.devAtomList_[k].molIndex_; }
    w.i("atom_type", type); w.i("atom_mol", mol);

    // Global bonded lists in the reference's discovery order (MolTwisterStateTools getAllMD*InSystem).
    {
        std::vector<int> b1, b2, bt, a1, a2, a3, at, d1, d2, d3, d4, dt;
        CMolTwisterStateTools tools(&st, stdout);
        tools.getAllMDBondsInSystem(b1, b2, bt, true);
        tools.getAllMDAnglesInSystem(a1, a2, a3, at, true);
        tools.getAllMDDihedralsInSystem(d1, d2, d3, d4, dt, true);
        std::vector<int32_t> B, A, D;
        for(size_t j = 0; j < b1.size(); j++) { B.push_back(b1[j]); B.push_back(b2[j]); B.push_back(bt[j]); }
        for(size_t j = 0; j < a1.size(); j++) { A.push_back(a1[j]); A.push_back(a2[j]); A.push_back(a3[j]); A.push_back(at[j]); }
        for(size_t j = 0; j < d1.size(); j++) { D.push_back(d1[j]); D.push_back(d2[j]); D.push_back(d3[j]); D.push_back(d4[j]); D.push_back(dt[j]); }
        w.i("bonds", B, {(uint64_t)b1.size(), 3}); w.i("angles", A, {(uint64_t)a1.size(), 4}); w.i("dihedrals", D, {(uint64_t)d1.size(), 5});
    }
    // Per-atom bonded lists (MDFFMatrices.cpp:384-520)
    {
        std::vector<int32_t> bp, bl, ap, al, dp, dl;
        for(int k = 0; k < N; k++) { bp.push_back(M.devBondsForAtomListPointers_[k].indexFirstEntry_); bp.push_back(M.devBondsForAtomListPointers_[k].numEntries_); }
        for(const auto& b : M.devBondsForAtomLists_) { bl.push_back((int)b.atomIndex1_); bl.push_back((int)b.atomIndex2_); bl.push_back(b.bondType_); }
        for(int k = 0; k < N; k++) { ap.push_back(M.devAnglesForAtomListPointers_[k].indexFirstEntry_); ap.push_back(M.devAnglesForAtomListPointers_[k].numEntries_); }
        for(const auto& a : M.devAnglesForAtomLists_) { al.push_back((int)a.atomIndex1_); al.push_back((int)a.atomIndex2_); al.push_back((int)a.atomIndex3_); al.push_back(a.angleType_); al.push_back(a.assocAtomIsAtCenterOfAngle_ ? 1 : 0); }
        for(int k = 0; k < N; k++) { dp.push_back(M.devDihedralsForAtomListPointers_[k].indexFirstEntry_); dp.push_back(M.devDihedralsForAtomListPointers_[k].numEntries_); }
        for(const auto& d : M.devDihedralsForAtomLists_) { dl.push_back((int)d.atomIndex1_); dl.push_back((int)d.atomIndex2_); dl.push_back((int)d.atomIndex3_); dl.push_back((int)d.atomIndex4_); dl.push_back(d.dihedralType_); dl.push_back(d.assocAtomIsAtCenterOfDihedral_ ? 1 : 0); }
        w.i("atom_bond_ptr", bp, {(uint64_t)N, 2}); w.i("atom_bonds", bl, {(uint64_t)bl.size() / 3, 3});
        w.i("atom_angle_ptr", ap, {(uint64_t)N, 2}); w.i("atom_angles", al, {(uint64_t)al.size() / 5, 5});
        w.i("atom_dih_ptr", dp, {(uint64_t)N, 2}); w.i("atom_dihs", dl, {(uint64_t)dl.size() / 6, 6});
    }

    // Cell list + neighbour list at the input positions (MDFFMatrices.cpp:151-179)
    std::vector<CParticle3D> P = particlesFromState(st);
    M.updateAtomList(P);
    M.genNeighList((float)s.L[0], (float)s.L[1], (float)s.L[2]);
    {
        std::vector<int32_t> ci, cp, cl, nc, nl;
        for(const auto& c : M.cellList_.devAtomCellIndices_) { ci.push_back(c.ix_); ci.push_back(c.iy_); ci.push_back(c.iz_); }
        for(const auto& p : M.cellList_.devCellListEntryPointers_) { cp.push_back(p.indexFirstEntry_); cp.push_back(p.numEntries_); }
        for(int v : M.cellList_.devCellList_) cl.push_back(v);
        for(int v : M.neighList_.devNeighListCount_) nc.push_back(v);
        for(int v : M.neighList_.devNeighList_) nl.push_back(v);
        const int maxN = M.neighList_.getMaxNeighbors();
        w.i("cell_dims", {M.cellList_.getCellCountX(), M.cellList_.getCellCountY(), M.cellList_.getCellCountZ()});
        w.i("atom_cell", ci, {(uint64_t)N, 3}); w.i("cell_ptr", cp, {(uint64_t)cp.size() / 2, 2}); w.i("cell_list", cl);
        w.i("neigh_count", nc); w.i("neigh_max", {maxN}); w.i("neigh_list", nl, {(uint64_t)N, (uint64_t)maxN});
    }

    // Forces through the public CVelVerlet entry (Integrators/VelVerlet.cpp:152-158)
    CVelVerlet vv(&st, stdout, cfg.cutoffRadius_, cfg.neighListShell_, cfg.cutoffForce_);
    vv.setNonBondedScaleFactors((float)cfg.scale12Interactions_, (float)cfg.scale13Interactions_,
                                (float)cfg.scale14Interactions_, (float)cfg.scaleAbove14BondedInteractions_);
    std::vector<CMDFFMatrices::CForces> F = vv.calcParticleForces(3, s.L[0], s.L[1], s.L[2], P);
    dumpForces(w, "", F);
    return 0;
}

// ------------------------------------------------------------------------------------------------
// run / time: CSimulationBox + MDLoop step sequence with injected initial state
// ------------------------------------------------------------------------------------------------
void injectState(const SysIn& s, CSimulationBox& sb) {
    const int N = sb.N_;
    if(!s.p.empty()) for(int k = 0; k < N; k++) sb.particles_[k].p_ = C3DVector(s.p[3 * k], s.p[3 * k + 1], s.p[3 * k + 2]);
    for(size_t j = 0; j < s.nhT_eta.size() && j < sb.NH_T_.eta_.size(); j++) sb.NH_T_.eta_[j] = s.nhT_eta[j];
    for(size_t j = 0; j < s.nhT_peta.size() && j < sb.NH_T_.p_eta_.size(); j++) sb.NH_T_.p_eta_[j] = s.nhT_peta[j];
    for(size_t j = 0; j < s.nhP_eta.size() && j < sb.NH_P_.eta_.size(); j++) sb.NH_P_.eta_[j] = s.nhP_eta[j];
    for(size_t j = 0; j < s.nhP_peta.size() && j < sb.NH_P_.p_eta_.size(); j++) sb.NH_P_.p_eta_[j] = s.nhP_peta[j];
    if(s.has_peps) sb.velVerlet_.p_eps_ = s.p_eps;
}

int cmdRun(const SysIn& s, const std::string& out, int nsteps, int stride) {
    CMolTwisterState st; buildState(s, st);
    SMolDynConfigStruct cfg = makeCfg(s);
    FILE* devnull = fopen("/dev/null", "w");
    COut::setStdOut(devnull);
    CSimulationBox sb(&st, devnull, cfg);
    injectState(s, sb);
    CFctT fctT(&sb);
    CFctP fctP(&sb.velVerlet_);
    C3DVector boxOut;
    const int N = sb.N_;
    std::vector<double> R, Pm, Fo, scal, nh, nhp, baro;
    std::vector<float> Uo;
    std::vector<CMDFFMatrices::CForces> F = sb.calcParticleForces();
    auto record = [&](int t) {
        for(int k = 0; k < N; k++) {
            R.push_back(sb.particles_[k].r_.x_); R.push_back(sb.particles_[k].r_.y_); R.push_back(sb.particles_[k].r_.z_);
            Pm.push_back(sb.particles_[k].p_.x_); Pm.push_back(sb.particles_[k].p_.y_); Pm.push_back(sb.particles_[k].p_.z_);
            Fo.push_back(F[k].F_.x_); Fo.push_back(F[k].F_.y_); Fo.push_back(F[k].F_.z_);
            Uo.push_back(F[k].U_);
        }
        // MDLoop.cpp:388-403: U, K, T, P, V
        scal.push_back((double)t);
        scal.push_back(sb.calcUtot(F));
        scal.push_back(sb.calcCurrentKineticEnergy());
        scal.push_back(sb.calcTemp());
        scal.push_back(sb.calcPress(F));
        scal.push_back(sb.calcV());
        for(int j = 0; j < sb.NH_T_.M_; j++) nh.push_back(sb.NH_T_.eta_[j]);
        for(int j = 0; j < sb.NH_T_.M_; j++) nh.push_back(sb.NH_T_.p_eta_[j]);
        for(int j = 0; j < sb.NH_P_.M_; j++) nhp.push_back(sb.NH_P_.eta_[j]);
        for(int j = 0; j < sb.NH_P_.M_; j++) nhp.push_back(sb.NH_P_.p_eta_[j]);
        baro.push_back(sb.velVerlet_.p_eps_);
    };
    record(-1);
    int nrec = 1;
    for(int t = 0; t < nsteps; t++) {
        sb.NHPPropagator(fctP);
        sb.NHTPropagator(fctT);
        sb.velVerPropagator(F, boxOut);
        sb.NHTPropagator(fctT);
        sb.NHPPropagator(fctP);
        sb.pbcWrap();
        if(((t + 1) % stride) == 0 || t == nsteps - 1) { record(t); nrec++; }
    }
    MtbWriter w(out);
    w.d("traj_r", R, {(uint64_t)nrec, (uint64_t)N, 3});
    w.d("traj_p", Pm, {(uint64_t)nrec, (uint64_t)N, 3});
    w.d("traj_F", Fo, {(uint64_t)nrec, (uint64_t)N, 3});
    w.f("traj_U", Uo, {(uint64_t)nrec, (uint64_t)N});
    w.d("traj_scalars", scal, {(uint64_t)nrec, 6});
    w.d("traj_nhT", nh, {(uint64_t)nrec, 2, (uint64_t)sb.NH_T_.M_});
    w.d("traj_nhP", nhp, {(uint64_t)nrec, 2, (uint64_t)sb.NH_P_.M_});
    w.d("traj_peps", baro, {(uint64_t)nrec});
    fclose(devnull);
    return 0;
}

// dcd: two DCD records (the input positions and the positions shifted by +0.125 A) written
// through the reference's CDCDFile::createDCDFileIfNotExists / appendToDCDFile
// (Utilities/DCDFile.cpp:670-729), as CMDLoop::appendToDCDFile calls them (MDLoop.cpp:248-258).
int cmdDcd(const SysIn& s, const std::string& out, int nsteps, int stride, double dt) {
    const int N = (int)s.atoms.size();
    remove(out.c_str());
    for(int rec = 0; rec < 2; rec++) {
        const double sh = 0.125 * rec;
        std::function<std::tuple<double, double, double>(const int&)> pos = [&s, sh](const int& i) -> std::tuple<double, double, double> {
            const AtomIn& a = s.atoms[i];
            return std::tuple<double, double, double>(a.x + sh, a.y + sh, a.z + sh);
        };
        CDCDFile::createDCDFileIfNotExists(out, nsteps, stride, dt, N);
        CDCDFile::appendToDCDFile(out, N, {s.L[0], s.L[1], s.L[2]}, pos);
    }
    return 0;
}

int cmdTime(const SysIn& s, int nsteps) {
    CMolTwisterState st; buildState(s, st);
    SMolDynConfigStruct cfg = makeCfg(s);
    FILE* devnull = fopen("/dev/null", "w");
    COut::setStdOut(devnull);
    CSimulationBox sb(&st, devnull, cfg);
    injectState(s, sb);
    CFctT fctT(&sb);
    CFctP fctP(&sb.velVerlet_);
    C3DVector boxOut;
    std::vector<CMDFFMatrices::CForces> F = sb.calcParticleForces();
    auto t0 = std::chrono::steady_clock::now();
    for(int t = 0; t < nsteps; t++) {
        sb.NHPPropagator(fctP);
        sb.NHTPropagator(fctT);
        sb.velVerPropagator(F, boxOut);
        sb.NHTPropagator(fctT);
        sb.NHPPropagator(fctP);
        sb.pbcWrap();
    }
    double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("{\"atoms\": %d, \"steps\": %d, \"seconds\": %.6f, \"utot\": %.17g}\n", sb.N_, nsteps, sec, sb.calcUtot(F));
    fclose(devnull);
    return 0;
}

// paircorr: `calculate paircorrelation` (Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.cpp) on a
// DCD file of nframes frames (frame f: the input positions shifted by f * shift on every axis),
// written through the reference's CDCDFile with the box truncated to integers as the MD loop
// writes it (MDLoop.cpp:248-258).  The command's table goes to OUT; the PBC widths it used for
// each frame (CDCDFile::getCurrentPBC) are appended as "pbc <f> <wx> <wy> <wz>" lines.
int cmdPairCorr(const SysIn& s, const std::string& out, int nframes, double shift, const std::vector<std::string>& args) {
    CMolTwisterState st; buildState(s, st);
    const int N = (int)s.atoms.size();
    const std::string dcd = out + ".dcd";
    remove(dcd.c_str());
    for(int f = 0; f < nframes; f++) {
        const double sh = shift * f;
        std::function<std::tuple<double, double, double>(const int&)> pos = [&s, sh](const int& i) -> std::tuple<double, double, double> {
            const AtomIn& a = s.atoms[i];
            return std::tuple<double, double, double>(a.x + sh, a.y + sh, a.z + sh);
        };
        CDCDFile::createDCDFileIfNotExists(dcd, nframes, 1, 1.0, N);
        CDCDFile::appendToDCDFile(dcd, N, {(int)s.L[0], (int)s.L[1], (int)s.L[2]}, pos);
    }
    FILE* fo = fopen(out.c_str(), "w");
    FILE* devnull = fopen("/dev/null", "w");
    COut::setStdOut(devnull);
    CCmdPairCorrelation cmd(&st, fo);
    std::vector<std::string> a = {dcd, "0", std::to_string(nframes)};
    a.insert(a.end(), args.begin(), args.end());
    const std::string err = cmd.execute(a);
    CDCDFile file;
    if(file.open(dcd)) {
        for(int f = 0; f < nframes; f++) {
            file.gotoRecord(f);
            const C3DRect pbc = file.getCurrentPBC();
            fprintf(fo, "pbc %d %.17g %.17g %.17g\n", f, pbc.getWidthX(), pbc.getWidthY(), pbc.getWidthZ());
        }
    }
    fclose(fo);
    fclose(devnull);
    remove(dcd.c_str());
    if(!err.empty()) {
        fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    return 0;
}

// desc: the descriptors the adapter (adapter.cpp) builds from the reference's objects
int cmdDesc(const SysIn& s, const std::string& out) {
    CMolTwisterState st; buildState(s, st);
    SMolDynConfigStruct cfg = makeCfg(s);
    FILE* devnull = fopen("/dev/null", "w");
    COut::setStdOut(devnull);
    mtgpu_adapter::Descriptors d;
    std::string err;
    if(!mtgpu_adapter::build(&st, cfg, d, err)) {
        fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    auto terms = [](const std::vector<mtg_term>& v, std::vector<int32_t>& kind, std::vector<double>& p) {
        for(const mtg_term& t : v) {
            kind.push_back(t.kind);
            for(int k = 0; k < 4; k++) p.push_back(t.p[k]);
        }
    };
    std::vector<int32_t> nk, bk, ak, dk;
    std::vector<double> np_, bp, ap, dp;
    terms(d.nb_terms, nk, np_);
    terms(d.bond_terms, bk, bp);
    terms(d.angle_terms, ak, ap);
    terms(d.dih_terms, dk, dp);
    std::vector<int32_t> mob(d.mobile.begin(), d.mobile.end());
    const mtg_config_desc& c = d.cfg;
    std::vector<double> cfgv = {(double)c.ensemble, (double)c.temperature_nh_len, (double)c.temperature_respa,
                                (double)c.pressure_nh_len, (double)c.pressure_respa, c.timestep, c.temperature,
                                c.temperature_relax, c.pressure, c.pressure_relax, c.cutoff_radius, c.neigh_shell,
                                c.cutoff_force, c.scale12, c.scale13, c.scale14, c.scale1N};
    MtbWriter w(out);
    w.d("r", d.r); w.d("mass", d.mass); w.d("charge", d.charge); w.i("type", d.type); w.i("mol", d.mol); w.i("mobile", mob);
    w.d("box", {d.sys.box[0], d.sys.box[1], d.sys.box[2]});
    w.i("nb_count", d.nb_count); w.i("nb_kind", nk); w.d("nb_p", np_); w.f("nb_tables", d.nb_tables);
    w.i("bond_kind", bk); w.d("bond_p", bp); w.f("bond_tables", d.bond_tables);
    w.i("angle_kind", ak); w.d("angle_p", ap); w.f("angle_tables", d.angle_tables);
    w.i("dih_kind", dk); w.d("dih_p", dp); w.f("dih_tables", d.dih_tables);
    w.i("bonds", d.bonds); w.i("angles", d.angles); w.i("dihedrals", d.dihedrals);
    w.d("cfg", cfgv);
    fclose(devnull);
    return 0;
}

// init: the initial state the reference's CSimulationBox constructor draws (initSystem,
// SimulationBox.cpp:53-96) after srand(seed); seed 1 is also what a fresh process draws with
int cmdInit(const SysIn& s, const std::string& out, unsigned seed) {
    CMolTwisterState st; buildState(s, st);
    SMolDynConfigStruct cfg = makeCfg(s);
    FILE* devnull = fopen("/dev/null", "w");
    COut::setStdOut(devnull);
    srand(seed);
    CSimulationBox sb(&st, devnull, cfg);
    const int N = sb.N_;
    std::vector<double> Pm, nh, nhp, peps;
    for(int k = 0; k < N; k++) {
        Pm.push_back(sb.particles_[k].p_.x_); Pm.push_back(sb.particles_[k].p_.y_); Pm.push_back(sb.particles_[k].p_.z_);
    }
    for(int j = 0; j < sb.NH_T_.M_; j++) nh.push_back(sb.NH_T_.eta_[j]);
    for(int j = 0; j < sb.NH_T_.M_; j++) nh.push_back(sb.NH_T_.p_eta_[j]);
    for(int j = 0; j < sb.NH_P_.M_; j++) nhp.push_back(sb.NH_P_.eta_[j]);
    for(int j = 0; j < sb.NH_P_.M_; j++) nhp.push_back(sb.NH_P_.p_eta_[j]);
    peps.push_back(sb.velVerlet_.p_eps_);
    MtbWriter w(out);
    w.d("init_p", Pm, {(uint64_t)N, 3});
    w.d("init_nhT", nh, {2, (uint64_t)sb.NH_T_.M_});
    w.d("init_nhP", nhp, {2, (uint64_t)sb.NH_P_.M_});
    w.d("init_peps", peps, {1});
    fclose(devnull);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if(argc < 3) {
        fprintf(stderr, "usage: mtref static SYS OUT | run SYS OUT NSTEPS STRIDE | time SYS NSTEPS | dcd SYS OUT NSTEPS STRIDE DT | init SYS OUT SEED | paircorr SYS OUT NFRAMES SHIFT ARGS... | desc SYS OUT\n");
        return 1;
    }
    std::string cmd = argv[1];
    SysIn s = readSys(argv[2]);
    if(cmd == "static" && argc >= 4) return cmdStatic(s, argv[3]);
    if(cmd == "run" && argc >= 6) return cmdRun(s, argv[3], atoi(argv[4]), atoi(argv[5]));
    if(cmd == "time" && argc >= 4) return cmdTime(s, atoi(argv[3]));
    if(cmd == "dcd" && argc >= 7) return cmdDcd(s, argv[3], atoi(argv[4]), atoi(argv[5]), atof(argv[6]));
    if(cmd == "init" && argc >= 5) return cmdInit(s, argv[3], (unsigned)strtoul(argv[4], nullptr, 10));
    if(cmd == "desc" && argc >= 4) return cmdDesc(s, argv[3]);
    if(cmd == "paircorr" && argc >= 6) {
        std::vector<std::string> rest(argv + 6, argv + argc);
        return cmdPairCorr(s, argv[3], atoi(argv[4]), atof(argv[5]), rest);
    }
    fprintf(stderr, "bad arguments\n");
    return 1;
}
