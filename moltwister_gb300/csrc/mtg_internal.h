// Internal declarations shared by the translation units of libmtgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/mtgpu.h"

namespace mtg {

constexpr int kNpts = MTG_NPTS;
constexpr int kMaxFF = MTG_MAX_FF_PER_PAIR;
constexpr int kMaxChain = MTG_MAX_NH_CHAIN;
constexpr float kCoulombKf = 1389.32f;     // Integrators/Constants.h:40 (float literal)
constexpr double kConvT = 120.272;         // Constants.h Conv_T
constexpr double kConvt = 1.0E2;           // Constants.h Conv_t
constexpr double kConvPress = 16388.2461;  // Constants.h Conv_press
// Fixed-point scale of the mixed-precision force and energy accumulators: 2^26 units per kJ/mol(/A).
constexpr double kFixScale = 67108864.0;   // 2^26
constexpr float kFixScaleF = 67108864.0f;
// Neighbour-list entry: atom index in the low 29 bits, exclusion class in the top 3 bits.
constexpr uint32_t kIdxMask = 0x1FFFFFFFu;
constexpr int kClassShift = 29;
// Exclusion classes (FunctorCalcForce.cpp:95-157): 0 none, 1 1-2, 2 1-3, 3 1-4, 4 same molecule.

// A double-float value hi + lo (two FP32 numbers, |lo| <= ulp(hi)/2): about 48 bits of mantissa
// from FP32 arithmetic.
struct DF {
    float h, l;
};

// Constants of the mixed-precision integration kernels for one system's box (NVT/NVE: fixed for
// the context's life), converted from FP64 once on the host instead of by every block.
struct MixConst {
    DF dt, dt2, fcut;
    DF conv[3], L[3];          // 2^32 / L, L
    float Lf[3], iLf[3], L2f[3];
    float h2, fcutf;           // (skin / 2)^2; cutoff force
    long long fcut_q;          // cutoff force in fixed point
};

// Device-side thermostat state.  `th` is the live chain; `saved` is the chain right after the
// second half-step of the last completed step (what the reference holds between steps).
struct ThermoDev {
    double eta[kMaxChain];
    double peta[kMaxChain];
    double Q[kMaxChain];
    double iQ[kMaxChain];   // 1/Q
};

// Barostat state of the NPT ensemble (CVelVerlet p_eps_, eps_, W_, V0_, P_: VelVerlet.h:57-62,
// SimulationBox.cpp:73-76) and the per-step coefficients derived from it.  `saved` fields hold the
// state after the last completed step; the live fields run one half-step ahead (the next step's
// barostat kick, strain update and box are computed at the end of the previous step).
struct BaroDev {
    double p_eps, eps;
    double L[3];          // current box getSimBox() (VelVerlet.cpp:198-211)
    float Lf[3];          // (float) L, what the list and force kernels use
    float pad0;
    double ap, bp;        // prop_p: p = p ap + F bp (VelVerlet.cpp:124-136)
    double ar, br;        // prop_r: r = r ar + (p (1/m)) br (VelVerlet.cpp:138-150)
    double p_eps_saved, eps_saved;
    double L_saved[3];
    // production modes: the current box as the production kernels read it (in place of the
    // Params fields), and what the Verlet list needs when the box changes between rebuilds
    double conv[3];       // 2^32 / L: box fractions of the mixed mode
    float fscale[3];      // L / 2^32
    float sb;             // L / Lb: scale of the box since the last list build
    double Lb[3];         // box at the last list build
    float h2;             // squared displacement that triggers a rebuild in the current box
    int pn[3];            // production cell counts for the current box (at most the allocated grid)
};

// One replica of a batch (several independent systems advanced by the same launches): its atom
// range, the block range of the 256-atom blocks of the integration kernels, its production cell
// grid (global cell indices cbase ..), box and cutoffs, and its temperature.
struct RepDev {
    int off, n;
    int bbase, nb;
    int cbase, pnx, pny, pnz;
    double box[3];
    double fconv[3];      // 2^32 / L
    float fscale[3];      // L / 2^32
    float rc, rcoul, skin;
    double kT;
};

// Scalars the step kernels exchange through device memory.
struct StepScalars {
    double S;             // pending momentum scale: c2(previous step) * c1(this step)
    double c2;            // scale of the last second half-step (applied on output / at run end)
    double KE2;           // sum p^2/m after the last second half-step (p scaled by c2)
    double U;             // total potential energy (output steps)
    double virial;        // sum F.r with wrapped r (output steps)
    int32_t rebuild;      // production list: 1 = rebuild before the next force evaluation
    int32_t overflow;     // list capacity exceeded (entries needed in `needed`)
    int32_t needed;
    int32_t nonfinite;
    uint32_t done_blocks; // last-block counter of the reduction kernels
    int32_t builds;       // neighbour-list rebuilds performed
    int32_t timeout;      // a bounded device wait gave up
    int32_t boxerr;       // NPT (production): the box shrank until a cutoff reached half its width
    int32_t builds_run;   // production list builds since the start of the current run
};

struct Params {
    int n, T;
    double box[3];
    float boxf[3];
    int ensemble, precision, coulomb, clip;
    double dt;            // reduced time step
    double kT;            // reduced temperature
    double tau;
    int M, nresp;
    double fcut;
    float rc, shell;
    float rcoul;          // Coulomb cutoff (production, cutoff mode)
    float skin;
    float scale[5];       // by exclusion class: 1, s12, s13, s14, s1N
    float scale12, scale13, scale14, scale1N;
    int nx, ny, nz;       // reference cell counts (from the input box, MDFFMatrices.cpp:56-58)
    int pnx, pny, pnz;    // production cell counts (cell edge >= rlist), 1 = all-pairs build
    int team;             // lanes per atom in the production force gather (8, 16, 32)
    float fscale[3];      // L / 2^32: fixed-point position unit per axis (mixed)
    double fconv[3];      // 2^32 / L
    int qtype;            // 1: charges are a function of the type (qtype table)
    int qon;              // 1: cutoff Coulomb with some charge nonzero (production); 0: no Coulomb work
    int qany;             // 1: some charge nonzero (reference precision: the all-pairs Coulomb kernel runs)
    int lj_shift;         // 0 truncated LJ, 1 energy shifted at the cutoff, 2 force shifted
    int nrep;             // 0: one system; > 0: a batch of nrep replicas (RepDev table)
    int ncell_total;      // batch: production cells of all replicas
    int nblk_total;       // batch: 256-atom integration blocks of all replicas
    // NPT
    int MP, nrespP;       // barostat chain length and RESPA steps
    double Pext;          // pressure / Conv_press
    double W;             // barostat mass: kT tauP^2 (reference), 3 (N + 1) kT tauP^2 (production)
    double QP;            // barostat chain masses kT tauP^2
    double V0;            // LmaxX LmaxY LmaxZ
    int wait_polls;       // limit of the bounded device waits (thermostat hand-overs)
    double chain_stage[2];// production particle chain: the Suzuki-Yoshida stage lengths w0 dt / nresp
                          // and (1 - 2 w0) dt / nresp, w0 = 1 / (2 - 2^(1/3))
};



// Production NPT: the fields of b derived from its box b.L and the box b.Lb of the last list
// build, computed by the same code on the host (state set, creation) and on the device (end of
// every step).  A pair left out of the list at the build was at least rlist = r + skin apart in
// box fractions times Lb; after the box scales by s = L / Lb and two atoms moved by at most
// delta in the current box it is at least s rlist - 2 delta apart, so the list stays valid while
// delta <= (skin s + r (s - 1)) / 2 for every pair radius r <= rfull (the smallest margin is at
// r = rfull when s < 1 and at r = 0 when s > 1).  The kernels compare the displacement from the
// build positions scaled by s.  Cell counts follow the box, at most the allocated grid; one cell
// when fewer than three fit.  Returns false when a cutoff reaches half the box.
__host__ __device__ inline bool baro_box_fields(const Params& P, BaroDev& b) {
    const double rfull = (double)fmaxf(P.rc, P.coulomb != MTG_COULOMB_ALLPAIRS ? P.rcoul : 0.0f);
    const double rlist = rfull + (double)P.skin;
    const int cap[3] = {P.pnx, P.pny, P.pnz};
    bool ok = true;
    for(int a = 0; a < 3; a++) {
        b.Lf[a] = (float)b.L[a];
        b.conv[a] = 4294967296.0 / b.L[a];
        b.fscale[a] = (float)(b.L[a] / 4294967296.0);
        int pn = (int)floor(b.L[a] / rlist);
        if(pn > cap[a]) pn = cap[a];
        if(pn < 3) pn = 1;
        b.pn[a] = pn;
        if(2.0 * rfull >= b.L[a] || (pn > 1 && 2.0 * rlist > b.L[a])) ok = false;
    }
    const double sb = b.L[0] / b.Lb[0];
    const double margin = (double)P.skin * sb + rfull * (sb < 1.0 ? sb - 1.0 : 0.0);
    b.sb = (float)sb;
    b.h2 = margin > 0.0 ? (float)(0.25 * margin * margin) : -1.0f;
    return ok;
}

// Everything a force/integration kernel reads, as raw device pointers.
struct DevSys {
    int n, T;
    // reference & fp64 masters
    double* r;            // [3n]
    double* p;            // [3n]
    double* F;            // [3n]  FP64 forces (reference, fp64)
    double* U;            // [n]   per-atom energies
    double* W;            // [n]   per-atom virial (production modes: pair r.F once per pair, bonded terms)
    double* m;            // [n]
    double* qd;           // [n]   charges (double)
    float* qf;            // [n]   charges as float (CMDFFMatrices::CAtom::q_)
    int* type;
    int* mol;
    int* mobile;
    // tables (x, -dU/dx, U); nb layout [((row*T + col)*5 + ff)*1000 + pt]
    const float* nb_tab;
    const int* nb_cnt;
    const float* bond_tab;
    const float* angle_tab;
    const float* dih_tab;
    const int* nb_kind;
    const double* nb_par;     // [pair*5+ff][4]
    const float* nb_parf;     // [pair*5+ff][4] (FP32 copy)
    const double* nb_fs;      // [pair*5+ff] force at the LJ cutoff (force-shifted LJ), else 0
    const float* nb_fsf;
    // production list radius per type pair, before the skin: 0 no short-range term, FLT_MAX the
    // global cutoff, > 0 the pair's own LJ cutoff, < 0 the full list radius max(rc, rcoul)
    const float* pair_cut;
    const int* bond_kind;
    const double* bond_par;   // [type][4]; angles hold (k, theta0 [rad], toRad, 0)
    const float* bond_parf;   // FP32 copies for the mixed kernels
    const int* angle_kind;
    const double* angle_par;
    const float* angle_parf;
    const int* dih_kind;
    const double* dih_par;
    const float* dih_parf;
    // per-atom bonded lists (CSR)
    const int *bptr, *bj, *bt;
    const int *aptr, *ai, *aj, *at, *acen;
    const int *dptr, *di, *dj, *dl, *dt, *dcen;
    // 1 when every partner an exclusion could name (bonded, 1-3 and 1-4 lists) shares the atom's
    // molecule index (>= 0): a pair of different molecules then has no exclusion
    const int* excl_local;
    // reference cell & neighbour lists
    int* atom_cell;       // [3n]
    int* cell_first;      // [ncell]
    int* cell_count;      // [ncell]
    int* cell_cursor;     // [ncell]
    int* cell_list;       // [n]
    int* nbr_count;       // [n]
    int* nbr_list;        // [n * nbr_max]
    int nbr_max;
    int* nbr_count_nb;    // [n]  how many entries of nbr_list have a non-bonded term (null: not kept)
    int* nbr_list_nb;     // [n * nbr_max] those entries, in list order
    int* force_order;     // [n]  atoms by (type, index): the reference-precision gather's thread order
    // production (Verlet) list
    int* pcell_of;        // [n] production cell of each atom
    int* pcell_first;     // [pncell]
    int* pcell_count;     // [pncell]
    int* pcell_cursor;    // [pncell]
    int* pcell_list;      // [n] atoms in cell order: slot -> atom (identity before the first build)
    int* slot_of;         // [n] atom -> slot (inverse of pcell_list)
    uint32_t* vlist;      // [n * vmax] one row per slot; entries are slots of the partners
    int* vcount;          // [n] per slot
    const MixConst* mixk; // [1] or [nrep]: the mixed integrator's constants per system
    int* vsr;             // [n] per slot: the row's first vsr entries are pairs with short-range
                          //     terms, the rest pairs with Coulomb only
    int vmax;
    double* r_build;      // [3n] positions at the last build (displacement check)
    float4* rb4;          // [n]  the same in FP32 (displacement test), per atom
    float4* rb4s;         // [n]  the same per slot (list distances)
    // mixed
    float4* hi;           // [n] x,y,z hi, charge
    float4* lo;           // [n] x,y,z lo, type bits
    uint4* pq;            // [n] x,y,z as 32-bit fractions of the box (wrap = minimum image), type
    uint4* pqs;           // [n] the same per slot (cell order), refreshed wherever pq is written
    float4* ph;           // [n] mixed: momenta x,y,z hi, 1/m hi (double-float pairs with pl)
    float4* pl;           // [n] mixed: momenta x,y,z lo, 1/m lo
    const float* qtype;   // [T] charge of each type when every atom of a type has the same charge
    long long* Fx;        // [n] fixed-point forces (SoA)
    long long* Fy;
    long long* Fz;
    float* inv_m;         // [n]
    // reductions
    double* partial;      // [nblocks * 4]
    StepScalars* sc;
    ThermoDev* th;
    ThermoDev* th_saved;
    double* rec;          // output record ring [8]
    // batch of replicas (Params::nrep > 0)
    const int* rep_of;    // [n] replica of each atom
    const int* blk_rep;   // [blocks] replica of each 256-atom integration block
    const RepDev* reps;   // [nrep]
    StepScalars* rsc;     // [nrep] per-replica scale, energies, last-block counters
    ThermoDev* ths;       // [nrep] per-replica chains
    ThermoDev* ths_saved; // [nrep]
    double* rrec;         // [nrep * 8] per-replica output records
    // NPT
    BaroDev* baro;
    ThermoDev* thp;       // barostat chain (NH_P_)
    ThermoDev* thp_saved;
};

#ifdef __CUDACC__
__device__ __forceinline__ float box_f(const DevSys& d, const Params& P, int a) {
    return P.ensemble == MTG_NPT ? d.baro->Lf[a] : P.boxf[a];
}
__device__ __forceinline__ double box_d(const DevSys& d, const Params& P, int a) {
    return P.ensemble == MTG_NPT ? d.baro->L[a] : P.box[a];
}
#endif

// Kernel launchers (defined in ref_kernels.cu and md_kernels.cu).
// Reference mode
void launch_ref_cells(const DevSys& d, const Params& P, cudaStream_t s);
void launch_ref_neigh(const DevSys& d, const Params& P, cudaStream_t s);
void launch_ref_force(const DevSys& d, const Params& P, cudaStream_t s);
void launch_ref_kick_drift(const DevSys& d, const Params& P, cudaStream_t s);
void launch_ref_kick2(const DevSys& d, const Params& P, bool output, cudaStream_t s);
// Shared
// step kernels launched with programmatic dependent launch while a plain step graph is captured
void set_pdl_launch(bool on);
void launch_prologue(const DevSys& d, const Params& P, cudaStream_t s);
// Production modes
// use_cond: inside a conditional step graph, the last block sets `cond` to the rebuild decision
void launch_prod_kick_drift(const DevSys& d, const Params& P, cudaStream_t s, cudaGraphConditionalHandle cond = 0,
                            bool use_cond = false);
void launch_prod_build(const DevSys& d, const Params& P, bool force, cudaStream_t s);
void launch_prod_force(const DevSys& d, const Params& P, bool energy, cudaStream_t s);
// Second half of the step: the per-atom kick and block sums (kKick2Atoms) and, in mixed mode, the
// one-block-per-system step end with the thermostat chain (kKick2StepEnd; FP64 mode runs its chain
// in the last block of the per-atom kernel).
enum Kick2Parts { kKick2Atoms = 1, kKick2StepEnd = 2, kKick2All = 3 };
void launch_prod_kick2(const DevSys& d, const Params& P, bool output, cudaStream_t s, int parts = kKick2All);
// Mixed mode keeps positions and momenta as double-float pairs (hi/lo, ph/pl) plus the box
// fractions pq; the FP64 arrays r and p are the masters the host reads and writes.
enum SyncMode { kSyncToMaster = 0, kSyncFromMaster = 1, kSyncPositionsFromMaster = 2 };
void launch_prod_sync(const DevSys& d, const Params& P, SyncMode mode, cudaStream_t s);
void launch_prod_check_list(const DevSys& d, const Params& P, cudaStream_t s);   // flags a rebuild if positions moved
void launch_settle(const DevSys& d, const Params& P, cudaStream_t s);   // state after the completed step
// Up to kCopyMax device-to-device copies (8-byte multiples at 8-byte aligned addresses) in one
// launch: the chunk snapshot of the run loop and its rollback.
constexpr int kCopyMax = 32;
struct CopyTable {
    const unsigned long long* src[kCopyMax];
    unsigned long long* dst[kCopyMax];
    unsigned long long words[kCopyMax];
    int n;
};
void launch_copy_table(const CopyTable& t, cudaStream_t s);
// Chain (and, with set_baro, barostat) state written by a kernel from its arguments, so that a
// state write-back needs no synchronous copy.
struct ChainSet {
    double eta[kMaxChain], peta[kMaxChain];     // particle chain, M entries
    double etaP[kMaxChain], petaP[kMaxChain];   // barostat chain, MP entries
    int M, MP;
    int set_baro;
    BaroDev baro;
};
void launch_set_chains(const DevSys& d, const ChainSet& cs, cudaStream_t s);
void launch_prod_forces_to_double(const DevSys& d, const Params& P, cudaStream_t s);
void launch_gd_step(const DevSys& d, const Params& P, double lr, cudaStream_t s);
int reduction_blocks(int n);
int integration_blocks(const Params& P);   // blocks of the 256-atom integration kernels

// Adjoint kernels (adjoint.cu): tangents of the analytic forces and energies in FP64 dual numbers,
// the smeared pair correlation of two types and its position gradient, vector kernels.
struct AdjTangents {
    const double* vpos;       // [3n] position tangents, or null
    const double* nb_par_t;   // [T*T*5*4], or null
    const double* nb_fs_t;    // [T*T*5], or null
    const double* q_t;        // [n], or null
    const double* bond_par_t; // [ntypes*4], or null
    const double* angle_par_t;
    const double* dih_par_t;
};
struct AdjRdf {
    int ta, tb, nbins;
    double rmax, width;
};
void launch_force_tangent(const DevSys& d, const Params& P, const double* pos, const AdjTangents& t, double* Ft, double* Ut,
                          cudaStream_t s);
void launch_rdf_rows(const DevSys& d, const Params& P, const double* pos, const AdjRdf& r, double* rows, cudaStream_t s);
void launch_rdf_reduce(const double* rows, int n, int nbins, double* hist, cudaStream_t s);
void launch_rdf_adjoint(const DevSys& d, const Params& P, const double* pos, const AdjRdf& r, const double* cb, double* grad,
                        cudaStream_t s);
void launch_axpy(int n3, double a, const double* x, const double* scale, double* y, cudaStream_t s);
int dot_blocks(int n);
void launch_dot_blocks(int n, const double* x, const double* y, double* out, cudaStream_t s);
void launch_inv_mass(int n, const double* m, double* im, cudaStream_t s);
// out[s] = sum x[off[s] .. off[s+1]) for s < nseg, fixed order
void launch_segment_sums(const double* x, const int* off, int nseg, double* out, cudaStream_t s);
void launch_pair_hist(const double* pos, const int* ia, int na, const int* ib, int nb, const double* box, double rmin,
                      double rmax, int nbins, double ignore_below, unsigned long long* prof, cudaStream_t s);
// out[0] += w * sum_k x[k] y[k] (deterministic; part holds dot_blocks(n) partials)
void launch_dot_accum(int n, const double* x, const double* y, double w, double* part, double* out, cudaStream_t s);

// Initial momenta and chain / barostat state (init_state.cpp), MTG_INIT_* modes.
int draw_initial_state(int n, const double* mass, const uint8_t* mobile, const mtg_config_desc* cfg, uint32_t seed,
                       int mode, double* p, mtg_thermo_state* th);

// Host-side table generation (tables.cpp): out[npts*3] = (x, -dU/dx, U)
int profile_nonbonded(int kind, const double* p, float r0, float r1, int npts, float* out);
int profile_bond(int kind, const double* p, float r0, float r1, int npts, float* out);
int profile_angle(int kind, const double* p, float t0, float t1, int npts, float* out);
int profile_dihedral(int kind, const double* p, float t0, float t1, int npts, float* out);

}  // namespace mtg
