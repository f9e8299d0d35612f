// C ABI of libmtgpu.so (include/mtgpu.h): context lifetime, uploads, the step loop and the
// parity hooks.  Host code; the kernels live in ref_kernels.cu and md_kernels.cu.
//
// Step loop.  One MD step is the reference sequence (MDLoop.cpp:128-133) mapped to kernels:
//   kick+drift (first thermostat half-step folded in as a pending momentum scale)
//   -> [reference: cell list + neighbour list every step | production: Verlet list if due]
//   -> force gather -> clip + kick + pbc wrap + KE block sums -> the system's totals and the
//   thermostat's second half-step and the next step's first half-step (the last block of the kick
//   in the reference and fp64 modes, a one-block-per-system kernel in the mixed mode).
// Steps are captured into CUDA graphs, one chunk per output interval; the state at the start of
// a chunk is kept so that a chunk whose neighbour list overflowed is redone after growing it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "mtg_internal.h"

using namespace mtg;

namespace {

thread_local std::string g_create_error;

struct DeviceArena {
    std::vector<void*> ptrs;
    ~DeviceArena() { release(); }
    void release() {
        for(void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

}  // namespace

struct mtg_ctx {
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    Params P{};
    DevSys d{};
    mtg_config_desc cfg{};
    int ncell_ref = 0, ncell_prod = 0;
    int nblocks_red = 0;
    // host mirrors
    std::vector<double> h_mass;
    std::vector<int> h_type;
    // force-field parameters as given (for mtg_set_params / gradients)
    std::vector<mtg_term> h_nb_terms;          // [T*T*5]
    std::vector<int> h_nb_count;               // [T*T]
    std::vector<double> h_nb_coef;             // [T*T*5*4] device coefficients
    std::vector<double> h_nb_fs;               // [T*T*5] LJ force at the cutoff (force-shifted LJ)
    std::vector<double> h_bond_par, h_angle_par, h_dih_par;   // device layouts
    std::vector<int> h_bond_kind, h_angle_kind, h_dih_kind;
    std::vector<double> h_charge;
    std::vector<uint8_t> h_mobile;
    mtg_config_desc h_cfg{};
    bool has_tables = false;
    // buffers
    std::vector<void*> bufs;         // owned device allocations
    void* nbr_buf = nullptr;         // reference neighbour list (growable)
    void* nbr_nb_buf = nullptr;      // its entries with a non-bonded term (same capacity)
    void* vlist_buf = nullptr;       // production list (growable)
    // snapshot for chunk rollback
    struct Snap {
        void* dst;
        const void* src;
        size_t bytes;
    };
    std::vector<Snap> snaps;
    std::vector<void*> snap_bufs;
    // graphs keyed by (steps, output_at_end + 2 * form)
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    int generation = 0;
    bool forces_valid = false;
    // Step graph form of the production modes: 0 = plain capture (the list-build kernels run every
    // step and return at once when no rebuild is due), 1 = the list build under a conditional IF
    // node.  Which is faster depends on the system (on GB300 the IF node costs more than the
    // early-exit kernels of a 9,000-atom system), so the first two chunks of at least
    // kTuneSteps steps run one form each, timed, and the faster is kept.  Both forms run the
    // same kernels on the same data: the trajectory does not depend on the choice.
    bool conditional = true;          // IF nodes accepted by this driver
    bool team_retuned = false;        // force-gather team size re-timed at the first run
    int graph_form = -1;              // chosen form, -1 while measuring
    double form_us[2] = {0.0, 0.0};   // best device time per step of each form so far
    int form_n[2] = {0, 0};           // chunks timed in each form
    int last_form = 0;
    mtg_run_stats stats{};
    // output staging
    std::vector<double> h_r, h_p;
    // pinned double buffer of the output callback: the copies of output step k land in buffer
    // k % 2 while the next chunk is already queued, and the callback reads them while it runs
    double* pin_r[2] = {nullptr, nullptr};
    double* pin_p[2] = {nullptr, nullptr};
    cudaEvent_t ev_out[2] = {nullptr, nullptr};
    // pinned staging of the chain and barostat state a state read returns (queued with the
    // position and momentum copies, one synchronisation for all)
    struct ThermoStage {
        ThermoDev th, thp;
        BaroDev baro;
    };
    ThermoStage* pin_th = nullptr;
    // batch of replicas (P.nrep > 0)
    std::vector<int> rep_off;          // nrep + 1 atom offsets
    std::vector<double> h_rep_box;     // 3 per replica
    std::vector<double> h_rrec;        // nrep * 8 records of the last output step

    ~mtg_ctx() {
        for(auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
        for(void* p : bufs) cudaFree(p);
        for(void* p : snap_bufs) cudaFree(p);
        if(nbr_buf) cudaFree(nbr_buf);
        if(nbr_nb_buf) cudaFree(nbr_nb_buf);
        if(vlist_buf) cudaFree(vlist_buf);
        if(ev0) cudaEventDestroy(ev0);
        if(ev1) cudaEventDestroy(ev1);
        for(int b = 0; b < 2; b++) {
            if(pin_r[b]) cudaFreeHost(pin_r[b]);
            if(pin_p[b]) cudaFreeHost(pin_p[b]);
            if(ev_out[b]) cudaEventDestroy(ev_out[b]);
        }
        if(pin_th) cudaFreeHost(pin_th);
        if(stream) cudaStreamDestroy(stream);
    }
};

namespace {

int fail(mtg_ctx* c, int code, const std::string& msg) {
    if(c) c->err = msg;
    else g_create_error = msg;
    return code;
}

#define CUDA_TRY(ctx, call)                                                                        \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if(e_ != cudaSuccess) {                                                                    \
            (void)cudaGetLastError(); /* do not leave a stale error for the next caller */         \
            return fail((ctx), MTG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
        }                                                                                          \
    } while(0)

// A copy ordered after the work already queued on the context's stream and complete when it
// returns.  The stream is non-blocking, so a plain cudaMemcpy (legacy default stream) would
// neither wait for that work nor be waited for by it.
cudaError_t copy_now(mtg_ctx* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, c->stream);
    if(e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e;
}

template<class T>
int dalloc(mtg_ctx* c, T** out, size_t count) {
    void* p = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&p, bytes);
    if(e != cudaSuccess) return fail(c, MTG_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    cudaMemsetAsync(p, 0, bytes, c->stream);
    c->bufs.push_back(p);
    *out = (T*)p;
    return MTG_OK;
}

template<class T>
int upload(mtg_ctx* c, T** out, const T* host, size_t count) {
    int rc = dalloc(c, out, count);
    if(rc) return rc;
    if(count && host) CUDA_TRY(c, copy_now(c, *out, host, count * sizeof(T), cudaMemcpyHostToDevice));
    return MTG_OK;
}

bool finite_all(const double* a, size_t n) {
    for(size_t i = 0; i < n; i++)
        if(!std::isfinite(a[i])) return false;
    return true;
}

// Per-atom bonded lists in the reference's order (MDFFMatrices.cpp:384-520).
struct AtomLists {
    std::vector<int> bptr, bj, bt, aptr, ai, aj, at, acen, dptr, di, dj, dl, dt, dcen;
};

AtomLists build_atom_lists(int n, int nb, const int* bonds, int na, const int* angles, int nd, const int* dih) {
    AtomLists L;
    std::vector<std::vector<int>> bl(n), al(n), dl(n);
    for(int j = 0; j < nb; j++) {
        const int a = bonds[3 * j], b = bonds[3 * j + 1], t = bonds[3 * j + 2];
        if(t < 0) continue;
        bl[a].push_back(j);
        if(b != a) bl[b].push_back(j);
    }
    for(int j = 0; j < na; j++) {
        if(angles[4 * j + 3] < 0) continue;
        int s[3] = {angles[4 * j], angles[4 * j + 1], angles[4 * j + 2]};
        std::sort(s, s + 3);
        for(int q = 0; q < 3; q++)
            if(q == 0 || s[q] != s[q - 1]) al[s[q]].push_back(j);
    }
    for(int j = 0; j < nd; j++) {
        if(dih[5 * j + 4] < 0) continue;
        int s[4] = {dih[5 * j], dih[5 * j + 1], dih[5 * j + 2], dih[5 * j + 3]};
        std::sort(s, s + 4);
        for(int q = 0; q < 4; q++)
            if(q == 0 || s[q] != s[q - 1]) dl[s[q]].push_back(j);
    }
    L.bptr.assign(n + 1, 0);
    L.aptr.assign(n + 1, 0);
    L.dptr.assign(n + 1, 0);
    for(int k = 0; k < n; k++) {
        L.bptr[k + 1] = L.bptr[k] + (int)bl[k].size();
        for(int j : bl[k]) {
            const int a = bonds[3 * j], b = bonds[3 * j + 1];
            int to = -1;
            if(a == k) to = b;
            if(b == k) to = a;
            L.bj.push_back(to);
            L.bt.push_back(bonds[3 * j + 2]);
        }
        L.aptr[k + 1] = L.aptr[k] + (int)al[k].size();
        for(int j : al[k]) {
            const int a1 = angles[4 * j], a2 = angles[4 * j + 1], a3 = angles[4 * j + 2];
            int I = -1, J = -1, cen = 0;
            if(a1 == k) { I = a2; J = a3; }
            if(a2 == k) { cen = 1; I = a1; J = a3; }
            if(a3 == k) { I = a2; J = a1; }
            L.ai.push_back(I);
            L.aj.push_back(J);
            L.at.push_back(angles[4 * j + 3]);
            L.acen.push_back(cen);
        }
        L.dptr[k + 1] = L.dptr[k] + (int)dl[k].size();
        for(int j : dl[k]) {
            const int a1 = dih[5 * j], a2 = dih[5 * j + 1], a3 = dih[5 * j + 2], a4 = dih[5 * j + 3];
            int I = -1, J = -1, Lx = -1, cen = 0;
            if(a1 == k) { I = a2; J = a3; Lx = a4; }
            if(a2 == k) { cen = 1; I = a1; J = a3; Lx = a4; }
            if(a3 == k) { cen = 1; I = a4; J = a2; Lx = a1; }
            if(a4 == k) { I = a3; J = a2; Lx = a1; }
            L.di.push_back(I);
            L.dj.push_back(J);
            L.dl.push_back(Lx);
            L.dt.push_back(dih[5 * j + 4]);
            L.dcen.push_back(cen);
        }
    }
    return L;
}

// Cells per axis as CCellList::init computes them (MDFFMatrices.cpp:45-58).
int ref_cells(double L, double rc, double shell) {
    const float R = (float)rc + (float)shell;
    return (int)std::floor(double((float)L / R));
}

int grow_neighbors(mtg_ctx* c, int needed) {
    const int cap = needed + 10;     // the reference grows to need + 10 (MDFFMatrices.cpp:172-176)
    if(c->nbr_buf) cudaFree(c->nbr_buf);
    if(c->nbr_nb_buf) cudaFree(c->nbr_nb_buf);
    c->nbr_buf = c->nbr_nb_buf = nullptr;
    c->d.nbr_list = c->d.nbr_list_nb = nullptr;
    void *p, *q;
    cudaError_t e = cudaMalloc(&p, (size_t)c->P.n * cap * sizeof(int));
    if(e != cudaSuccess) return fail(c, MTG_E_NOMEM, "neighbour list allocation failed");
    c->nbr_buf = p;
    e = cudaMalloc(&q, (size_t)c->P.n * cap * sizeof(int));
    if(e != cudaSuccess) return fail(c, MTG_E_NOMEM, "neighbour list allocation failed");
    c->nbr_nb_buf = q;
    c->d.nbr_list = (int*)p;
    c->d.nbr_list_nb = (int*)q;
    c->d.nbr_max = cap;
    c->generation++;
    return MTG_OK;
}

// Production list radius per type pair before the skin (DevSys::pair_cut): 0 when the pair has no
// short-range term, its own LJ cutoff when every term of the pair has one, FLT_MAX (the global
// cutoff) otherwise.  Coulomb widens every pair to rcoul on the device when charges are on.  The
// pair (full_a, full_b) keeps the full list radius (a pair-correlation loss reads its pairs from
// the list).
std::vector<float> pair_cuts(const mtg_ctx* c, int full_a, int full_b) {
    const int T = c->P.T;
    std::vector<float> pc((size_t)T * T, 0.0f);
    for(int a = 0; a < T; a++)
        for(int b = 0; b < T; b++) {
            const int q = a * T + b;
            float v = 0.0f;
            for(int ff = 0; ff < c->h_nb_count[q]; ff++) {
                const mtg_term& t = c->h_nb_terms[(size_t)q * kMaxFF + ff];
                const bool own = (t.kind == MTG_NB_LJ || t.kind == MTG_NB_LJ1208) && t.p[3] > 0.0;
                v = own ? std::max(v, (float)t.p[3]) : FLT_MAX;
            }
            if((a == full_a && b == full_b) || (a == full_b && b == full_a)) v = -1.0f;
            pc[q] = v;
        }
    return pc;
}

int upload_pair_cuts(mtg_ctx* c, int full_a, int full_b) {
    const std::vector<float> pc = pair_cuts(c, full_a, full_b);
    CUDA_TRY(c, cudaMemcpyAsync((void*)c->d.pair_cut, pc.data(), sizeof(float) * pc.size(), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MTG_OK;
}

// 1 when the production kernels have Coulomb work: a cutoff mode and some nonzero charge.
int any_charge(const mtg_ctx* c) {
    for(double q : c->h_charge)
        if(q != 0.0) return 1;
    return 0;
}

int charges_on(const mtg_ctx* c) {
    if(c->P.coulomb == MTG_COULOMB_ALLPAIRS) return 0;
    return any_charge(c);
}

// Verlet list capacity per slot: a multiple of 32 (rows start on 128-byte boundaries), with 25 %
// headroom over `needed` unless `exact` asks for the smallest multiple of 32 holding it.
int grow_vlist(mtg_ctx* c, int needed, bool exact = false) {
    const int cap = exact ? (std::max(needed, 1) + 31) / 32 * 32 : ((needed + needed / 4 + 32) + 31) / 32 * 32;
    if(c->vlist_buf) cudaFree(c->vlist_buf);
    c->vlist_buf = nullptr;
    void* p;
    cudaError_t e = cudaMalloc(&p, (size_t)c->P.n * cap * sizeof(uint32_t));
    if(e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(c, MTG_E_NOMEM, "Verlet list allocation of " + std::to_string((size_t)c->P.n * cap * sizeof(uint32_t)) +
                                        " bytes failed: " + cudaGetErrorString(e));
    }
    c->vlist_buf = p;
    c->d.vlist = (uint32_t*)p;
    c->d.vmax = cap;
    c->generation++;
    return MTG_OK;
}

StepScalars read_scalars(mtg_ctx* c) {
    StepScalars s{};
    cudaMemcpyAsync(&s, c->d.sc, sizeof(s), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    return s;
}

void clear_overflow(mtg_ctx* c) {
    // zero overflow, needed, nonfinite (contiguous int32 fields) and the timeout flags (the
    // system's and, in a batch, each replica's): each chunk reports its own
    cudaMemsetAsync(&c->d.sc->overflow, 0, 3 * sizeof(int32_t), c->stream);
    cudaMemsetAsync(&c->d.sc->timeout, 0, 2 * sizeof(int32_t), c->stream);   // timeout, boxerr
    if(c->P.nrep) {
        cudaMemset2DAsync(&c->d.rsc[0].timeout, sizeof(StepScalars), 0, sizeof(int32_t), c->P.nrep, c->stream);
        cudaMemset2DAsync(&c->d.rsc[0].nonfinite, sizeof(StepScalars), 0, sizeof(int32_t), c->P.nrep, c->stream);
    }
}

bool is_reference(const mtg_ctx* c) { return c->P.precision == MTG_PREC_REFERENCE; }
bool is_mixed(const mtg_ctx* c) { return c->P.precision == MTG_PREC_MIXED; }

// Forces at the current positions, growing lists as needed.  Host-synchronous.
// keep_list: the production Verlet list is rebuilt only if an atom moved more than half the skin
// since the last build (positions written from the host; the box unchanged), else always.
int compute_forces_now(mtg_ctx* c, bool energy, bool keep_list = false) {
    for(int attempt = 0; attempt < 64; attempt++) {
        clear_overflow(c);
        if(is_reference(c)) {
            launch_ref_cells(c->d, c->P, c->stream);
            launch_ref_neigh(c->d, c->P, c->stream);
            launch_ref_force(c->d, c->P, c->stream);
        } else {
            // a redo after an overflow rebuilds whatever the test said (the failed build moved the
            // build positions)
            const bool test = keep_list && attempt == 0;
            if(test) launch_prod_check_list(c->d, c->P, c->stream);
            launch_prod_build(c->d, c->P, !test, c->stream);
            launch_prod_force(c->d, c->P, energy, c->stream);
        }
        CUDA_TRY(c, cudaGetLastError());
        StepScalars s = read_scalars(c);
        CUDA_TRY(c, cudaGetLastError());
        if(!s.overflow) {
            c->forces_valid = true;
            return MTG_OK;
        }
        int rc = is_reference(c) ? grow_neighbors(c, s.needed) : grow_vlist(c, s.needed);
        if(rc) return rc;
    }
    return fail(c, MTG_E_OVERFLOW, "neighbour list did not converge");
}

// Autotuner for the production force gather: times each team size (lanes per atom) on this
// system with CUDA events on the context's stream and keeps the fastest.  Choices are cached per
// (precision, atom-count bucket, list radius, density bucket) for the process.
struct TuneKey {
    int precision, nbucket, rlist10, rho100;
    bool operator<(const TuneKey& o) const {
        return std::tie(precision, nbucket, rlist10, rho100) < std::tie(o.precision, o.nbucket, o.rlist10, o.rho100);
    }
};
std::map<TuneKey, int> g_tuned;
std::mutex g_tuned_mutex;   // contexts may be created on several host threads at once

// `fresh` re-times even when the class has a cached choice (the first run of a context, when the
// configuration is the one that will run rather than an unrelaxed start) and stores the result.
// Each team size is timed in three interleaved rounds of five launches; its fastest round counts.
int autotune_force(mtg_ctx* c, bool fresh = false) {
    const Params& P = c->P;
    const double V = P.box[0] * P.box[1] * P.box[2];
    const double rlist = std::max((double)P.rc, P.coulomb != MTG_COULOMB_ALLPAIRS ? (double)P.rcoul : 0.0) + P.skin;
    TuneKey key{P.precision, (int)std::floor(std::log2((double)P.n)), (int)std::lround(rlist * 10.0), (int)std::lround(100.0 * P.n / V)};
    if(!fresh) {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        auto it = g_tuned.find(key);
        if(it != g_tuned.end()) {
            c->P.team = it->second;
            return MTG_OK;
        }
    }
    const int teams[3] = {8, 16, 32};
    float best_of[3] = {1e30f, 1e30f, 1e30f};
    for(int round = 0; round < 3; round++) {
        for(int k = 0; k < 3; k++) {
            c->P.team = teams[k];
            launch_prod_force(c->d, c->P, false, c->stream);
            CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
            for(int r = 0; r < 5; r++) launch_prod_force(c->d, c->P, false, c->stream);
            CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
            CUDA_TRY(c, cudaEventSynchronize(c->ev1));
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            best_of[k] = std::min(best_of[k], ms);
        }
    }
    int best_team = 32;
    float best = 1e30f;
    for(int k = 0; k < 3; k++) {
        if(best_of[k] < best) {
            best = best_of[k];
            best_team = teams[k];
        }
    }
    c->P.team = best_team;
    {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        g_tuned[key] = best_team;
    }
    // leave the forces of the chosen variant in place
    launch_prod_force(c->d, c->P, true, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    return MTG_OK;
}

int enqueue_step(mtg_ctx* c, bool output) {
    if(is_reference(c)) {
        launch_ref_kick_drift(c->d, c->P, c->stream);
        launch_ref_cells(c->d, c->P, c->stream);
        launch_ref_neigh(c->d, c->P, c->stream);
        launch_ref_force(c->d, c->P, c->stream);
        launch_ref_kick2(c->d, c->P, output, c->stream);
    } else {
        launch_prod_kick_drift(c->d, c->P, c->stream);
        launch_prod_build(c->d, c->P, false, c->stream);
        launch_prod_force(c->d, c->P, output, c->stream);
        launch_prod_kick2(c->d, c->P, output, c->stream);
    }
    return MTG_OK;
}

// Kernels per step when no list rebuild is due (reference mode rebuilds every step).
int kernels_per_step(const mtg_ctx* c) {
    // reference: kick-drift, four cell-list kernels, the neighbour list, bonded and short-range
    // force kernels (+ all-pairs Coulomb with charges), kick; production plain form: kick-drift,
    // six list-build kernels, force, kick (+ the step end in mixed mode); conditional form: the
    // build kernels only inside the IF node
    if(is_reference(c)) return 9 + (c->P.qany ? 1 : 0);
    return (c->last_form == 0 ? 9 : 3) + (is_mixed(c) ? 1 : 0);
}

constexpr int kTuneSteps = 20;

// Step graph form for the next chunk (see mtg_ctx::graph_form): the first four chunks of at least
// kTuneSteps steps alternate the two forms (conditional, plain, conditional, plain), and the form
// with the lower best time per step is kept.  List builds fall into the timed chunks of both forms
// alike; taking each form's best chunk keeps an unlucky one (more builds, a slow first launch)
// from deciding.
int choose_form(mtg_ctx* c, int steps) {
    if(is_reference(c) || !c->conditional) return 0;
    if(c->graph_form >= 0) return c->graph_form;
    if(steps < kTuneSteps) return 0;
    return ((c->form_n[0] + c->form_n[1]) % 2 == 0) ? 1 : 0;
}

void record_form(mtg_ctx* c, int form, int steps, float ms) {
    if(c->graph_form >= 0 || steps < kTuneSteps || is_reference(c)) return;
    if(!c->conditional) {
        c->graph_form = 0;
        return;
    }
    const double us = 1000.0 * ms / steps;
    c->form_us[form] = c->form_n[form] ? std::min(c->form_us[form], us) : us;
    c->form_n[form]++;
    if(c->form_n[0] >= 2 && c->form_n[1] >= 2) c->graph_form = (c->form_us[1] < c->form_us[0]) ? 1 : 0;
}

template<class F>
int capture_segment(mtg_ctx* c, cudaGraph_t* out, F&& body) {
    CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    body();
    cudaError_t e = cudaStreamEndCapture(c->stream, out);
    if(e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(c, MTG_E_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    }
    return MTG_OK;
}

// Production step graph with the list build under an IF node: each step is
//   child(kick+drift, sets the condition) -> IF(rebuild){ child(list build) } -> child(force, kick+reduce)
// assembled explicitly from captured segments.  Returns non-zero if the CUDA driver refuses conditional nodes.
int build_conditional_graph(mtg_ctx* c, int steps, bool output, cudaGraph_t* out) {
    cudaGraph_t G = nullptr, gC = nullptr, gCo = nullptr;
    int rc = MTG_OK;
    auto cleanup = [&]() {
        for(cudaGraph_t x : {gC, gCo}) if(x) cudaGraphDestroy(x);
    };
    CUDA_TRY(c, cudaGraphCreate(&G, 0));
    rc = rc || capture_segment(c, &gC, [&] {
        launch_prod_force(c->d, c->P, false, c->stream);
        launch_prod_kick2(c->d, c->P, false, c->stream);
    });
    rc = rc || capture_segment(c, &gCo, [&] {
        launch_prod_force(c->d, c->P, true, c->stream);
        launch_prod_kick2(c->d, c->P, true, c->stream);
    });
    if(rc) {
        cleanup();
        cudaGraphDestroy(G);
        return rc;
    }
    cudaGraphNode_t prev = nullptr;
    for(int s = 0; s < steps && !rc; s++) {
        // a conditional handle belongs to one IF node: each step has its own, set by its own
        // kick-drift kernel
        cudaGraphConditionalHandle cond;
        const char* where = "conditional handle";
        cudaError_t e = cudaGraphConditionalHandleCreate(&cond, G, 0, cudaGraphCondAssignDefault);
        cudaGraph_t gA = nullptr;
        if(e == cudaSuccess) {
            where = "kick-drift node";
            if(capture_segment(c, &gA, [&] { launch_prod_kick_drift(c->d, c->P, c->stream, cond, true); }) != MTG_OK)
                e = cudaErrorUnknown;
        }
        cudaGraphNode_t nA, nB, nC;
        if(e == cudaSuccess) e = cudaGraphAddChildGraphNode(&nA, G, prev ? &prev : nullptr, prev ? 1 : 0, gA);
        if(gA) cudaGraphDestroy(gA);
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        if(e == cudaSuccess) {
            where = "IF node";
            e = cudaGraphAddNode(&nB, G, &nA, nullptr, 1, &np);
        }
        if(e == cudaSuccess) {
            // the list build is captured straight into the IF node's body graph
            where = "list build in the IF body";
            cudaGraph_t body = np.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if(e == cudaSuccess) {
                launch_prod_build(c->d, c->P, false, c->stream);
                e = cudaStreamEndCapture(c->stream, &body);
            }
        }
        if(e == cudaSuccess) {
            where = "force node";
            e = cudaGraphAddChildGraphNode(&nC, G, &nB, 1, (output && s == steps - 1) ? gCo : gC);
        }
        if(e != cudaSuccess) {
            (void)cudaGetLastError();
            rc = fail(c, MTG_E_UNSUPPORTED, std::string("conditional step graph (") + where + "): " + cudaGetErrorString(e));
        }
        prev = nC;
    }
    cleanup();
    if(rc) {
        cudaGraphDestroy(G);
        return rc;
    }
    *out = G;
    return MTG_OK;
}

int get_graph(mtg_ctx* c, int steps, bool output, int form, cudaGraphExec_t* out) {
    if(form == 1 && !c->conditional) form = 0;
    auto key = std::make_pair(steps, (output ? 1 : 0) + 2 * form);
    auto it = c->graphs.find(key);
    if(it != c->graphs.end()) {
        *out = it->second;
        c->last_form = form;
        return MTG_OK;
    }
    cudaGraph_t g = nullptr;
    c->last_form = 0;
    if(form == 1 && !is_reference(c)) {
        if(build_conditional_graph(c, steps, output, &g) == MTG_OK) {
            cudaGraphExec_t ge;
            const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            g = nullptr;
            if(e == cudaSuccess) {
                cudaGraphUpload(ge, c->stream);   // not on the first timed launch
                c->graphs[key] = ge;
                *out = ge;
                c->last_form = 1;
                return MTG_OK;
            }
            (void)cudaGetLastError();
            c->err = std::string("conditional step graph (instantiation): ") + cudaGetErrorString(e);
        }
        c->conditional = false;   // IF nodes refused: plain capture (early-exit build kernels) from now on
        key = std::make_pair(steps, output ? 1 : 0);
    }
    CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    set_pdl_launch(!is_reference(c));
    for(int s = 0; s < steps; s++) enqueue_step(c, output && s == steps - 1);
    set_pdl_launch(false);
    CUDA_TRY(c, cudaStreamEndCapture(c->stream, &g));
    cudaGraphExec_t ge;
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if(e != cudaSuccess) return fail(c, MTG_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    cudaGraphUpload(ge, c->stream);
    c->graphs[key] = ge;
    *out = ge;
    return MTG_OK;
}

void drop_graphs(mtg_ctx* c) {
    for(auto& g : c->graphs) cudaGraphExecDestroy(g.second);
    c->graphs.clear();
}

int add_snap(mtg_ctx* c, const void* src, size_t bytes) {
    void* p;
    if(cudaMalloc(&p, std::max<size_t>(bytes, 1)) != cudaSuccess) return fail(c, MTG_E_NOMEM, "snapshot allocation failed");
    c->snap_bufs.push_back(p);
    c->snaps.push_back({p, src, bytes});
    return MTG_OK;
}

// The snapshot copies as one launch (the copies of a chunk's snapshot would otherwise cost a
// host call each before the chunk's graph can be queued); any copy that is not a whole number of
// 8-byte words goes through cudaMemcpyAsync.
void copy_snaps(mtg_ctx* c, bool take) {
    CopyTable t{};
    for(auto& s : c->snaps) {
        void* to = take ? s.dst : (void*)s.src;
        const void* from = take ? s.src : s.dst;
        const bool words = s.bytes % 8 == 0 && (reinterpret_cast<uintptr_t>(to) | reinterpret_cast<uintptr_t>(from)) % 8 == 0;
        if(!words || t.n == kCopyMax) {
            cudaMemcpyAsync(to, from, s.bytes, cudaMemcpyDeviceToDevice, c->stream);
            continue;
        }
        t.src[t.n] = static_cast<const unsigned long long*>(from);
        t.dst[t.n] = static_cast<unsigned long long*>(to);
        t.words[t.n] = s.bytes / 8;
        t.n++;
    }
    launch_copy_table(t, c->stream);
}

void take_snapshot(mtg_ctx* c) { copy_snaps(c, true); }

void restore_snapshot(mtg_ctx* c) {
    copy_snaps(c, false);
    // production NPT: the restored barostat state holds the box of an earlier list build than the
    // list in place, so the next step rebuilds it
    if(c->P.ensemble == MTG_NPT && !is_reference(c)) cudaMemsetAsync(&c->d.sc->rebuild, 0xff, sizeof(int32_t), c->stream);
}

// Host copies of r and p after a step; p carries the pending scale c2 of the last second
// thermostat half-step (the kernels apply it lazily at the next kick).
// Pending second-half scale c2 of each replica (one entry for a single system).
int replica_c2(mtg_ctx* c, std::vector<double>& c2) {
    if(!c->P.nrep) {
        c2.assign(1, read_scalars(c).c2);
        return MTG_OK;
    }
    std::vector<StepScalars> rs(c->P.nrep);
    CUDA_TRY(c, copy_now(c, rs.data(), c->d.rsc, sizeof(StepScalars) * rs.size(), cudaMemcpyDeviceToHost));
    c2.resize(rs.size());
    for(size_t r = 0; r < rs.size(); r++) c2[r] = rs[r].c2;
    return MTG_OK;
}

// A double rounded to the nearest double-float pair (hi = float(x), lo = float(x - hi)) and back,
// as the mixed mode stores a momentum the host scaled (k_sync, then the FP64 master from hi + lo).
double round_df(double x) {
    const float h = (float)x;
    return (double)h + (double)(float)(x - (double)h);
}

// Momenta times the pending thermostat scale c2 of their system; in the mixed mode the result is
// rounded as the device stores it, so an output record's momenta equal the state a run that ends
// at that step leaves.
void scale_momenta(mtg_ctx* c, std::vector<double>& p, const std::vector<double>& c2) {
    const bool df = is_mixed(c);
    if(!c->P.nrep) {
        if(c2[0] != 1.0)
            for(double& v : p) v = df ? round_df(v * c2[0]) : v * c2[0];
        return;
    }
    for(int r = 0; r < c->P.nrep; r++)
        if(c2[r] != 1.0)
            for(size_t i = (size_t)3 * c->rep_off[r]; i < (size_t)3 * c->rep_off[r + 1]; i++)
                p[i] = df ? round_df(p[i] * c2[r]) : p[i] * c2[r];
}

// One output step whose positions and momenta are on their way into pinned buffer `buf`.
struct PendingOutput {
    bool live = false;
    int buf = 0;
    int64_t step = 0;
    double rec[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    std::vector<double> c2;
};

// Queues the copies of r and p (with the pending thermostat scales read now) into pinned buffer
// `buf`; the caller delivers them once the next chunk is queued.
int queue_output(mtg_ctx* c, int buf, double c2, PendingOutput& out) {
    const size_t n3 = (size_t)c->P.n * 3;
    if(!c->pin_r[buf]) {
        CUDA_TRY(c, cudaMallocHost((void**)&c->pin_r[buf], n3 * sizeof(double)));
        CUDA_TRY(c, cudaMallocHost((void**)&c->pin_p[buf], n3 * sizeof(double)));
        CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_out[buf], cudaEventDisableTiming));
    }
    out.c2.assign(1, c2);
    if(c->P.nrep) {
        int rc = replica_c2(c, out.c2);
        if(rc) return rc;
    }
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncToMaster, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(c->pin_r[buf], c->d.r, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->pin_p[buf], c->d.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaEventRecord(c->ev_out[buf], c->stream));
    out.buf = buf;
    out.live = true;
    return MTG_OK;
}

// Waits for a queued output step's copies and calls the callback; *stop is its request to stop.
int deliver_output(mtg_ctx* c, PendingOutput& o, mtg_output_cb cb, void* user, bool* stop) {
    *stop = false;
    if(!o.live) return MTG_OK;
    o.live = false;
    CUDA_TRY(c, cudaEventSynchronize(c->ev_out[o.buf]));
    const size_t n3 = (size_t)c->P.n * 3;
    std::vector<double> pv(c->pin_p[o.buf], c->pin_p[o.buf] + n3);
    scale_momenta(c, pv, o.c2);
    std::memcpy(c->pin_p[o.buf], pv.data(), n3 * sizeof(double));
    mtg_output out{};
    out.step = o.step;
    out.U = o.rec[0];
    out.K = o.rec[1];
    out.T = o.rec[2];
    out.P = o.rec[3];
    out.V = o.rec[4];
    out.E = o.rec[0] + o.rec[1];
    out.r = c->pin_r[o.buf];
    out.p = c->pin_p[o.buf];
    *stop = cb(&out, user) != 0;
    return MTG_OK;
}

int fetch_rp(mtg_ctx* c, double c2) {
    const size_t n3 = (size_t)c->P.n * 3;
    c->h_r.resize(n3);
    c->h_p.resize(n3);
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncToMaster, c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(c->h_r.data(), c->d.r, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->h_p.data(), c->d.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    std::vector<double> sc(1, c2);
    if(c->P.nrep) {
        int rc = replica_c2(c, sc);
        if(rc) return rc;
    }
    scale_momenta(c, c->h_p, sc);
    return MTG_OK;
}

// Cutoff terms of a 12-6 / 12-8 LJ term with device coefficients co (a, b): the energy constant
// (mode 1: U(rc); mode 2: U(rc) + rc F(rc)) and the force at the cutoff F(rc) (mode 2), for the
// term's own cutoff or the global one.
void lj_shift_terms(const mtg_term& t, const double* co, double rc_global, int mode, double* ushift, double* fcut) {
    *ushift = 0.0;
    *fcut = 0.0;
    if(mode == 0) return;
    const double rct = t.p[3] > 0.0 ? t.p[3] : rc_global;
    const bool six = t.kind == MTG_NB_LJ;
    const double ir = 1.0 / rct, ir2 = ir * ir, ir4 = ir2 * ir2, ir6 = ir4 * ir2, irn = six ? ir6 : ir4 * ir4;
    const double Uc = co[0] * ir6 * ir6 - co[1] * irn;
    const double Fc = (12.0 * co[0] * ir6 * ir6 - (six ? 6.0 : 8.0) * co[1] * irn) * ir;
    if(mode == 1) {
        *ushift = Uc;
    } else {
        *ushift = Uc + rct * Fc;
        *fcut = Fc;
    }
}

// A batch of independent replicas merged into one system: atom ranges, boxes, temperatures.
struct BatchSpec {
    int nrep = 0;
    std::vector<int> off, n;          // nrep + 1 offsets, nrep sizes
    std::vector<double> box;          // 3 per replica
    std::vector<double> temperature;  // K per replica
    std::vector<double> cutoff;       // A per replica (LJ and Coulomb), empty = the shared cutoffs
};

// Barostat state with momentum p_eps and strain eps: box L = (V0 e^{3 eps} / Vmax)^{1/3} Lmax
// (VelVerlet.cpp:192-211); the saved copy equals the live one (no step pending).
DF host_df(double x) {
    DF r;
    r.h = (float)x;
    r.l = (float)(x - (double)r.h);
    return r;
}

// The mixed integrator's constants for a box, converted as the device's df_of would.
MixConst mix_const_for(const Params& P, const double* box, const double* fconv, float skin) {
    MixConst m{};
    m.dt = host_df(P.dt);
    m.dt2 = host_df(P.dt / 2.0);
    for(int a = 0; a < 3; a++) {
        m.conv[a] = host_df(fconv[a]);
        m.L[a] = host_df(box[a]);
        m.Lf[a] = (float)box[a];
        m.iLf[a] = (float)(1.0 / box[a]);
        m.L2f[a] = (float)(0.5 * box[a]);
    }
    const float hs = 0.5f * skin;
    m.h2 = hs * hs;
    m.fcut = host_df(P.fcut);
    m.fcutf = (float)P.fcut;
    m.fcut_q = (long long)(P.fcut * kFixScale);
    return m;
}

// Barostat state at strain eps (box L = (V0 e^{3 eps} / Vmax)^{1/3} Lmax, VelVerlet.cpp:198-211).
// `box`, when given, is that box as a previous get_state returned it: used as is when it agrees
// with eps to rounding, so that a state written back continues bit for bit.  The production modes
// also derive the box fields their kernels read, with the list counted as built in this box (the
// caller rebuilds it).  Returns false when a cutoff reaches half the box.
bool baro_at(const Params& P, double p_eps, double eps, BaroDev* out, const double* box = nullptr) {
    BaroDev b{};
    b.p_eps = b.p_eps_saved = p_eps;
    b.eps = b.eps_saved = eps;
    const double Vmax = P.box[0] * P.box[1] * P.box[2];
    double ec = (P.V0 * std::exp(3.0 * eps)) / Vmax;
    ec = std::pow(ec, 1.0 / 3.0);
    for(int a = 0; a < 3; a++) {
        b.L[a] = (eps == 0.0) ? P.box[a] : ec * P.box[a];
        if(box && std::fabs(box[a] - b.L[a]) <= 1e-12 * b.L[a]) b.L[a] = box[a];
        b.L_saved[a] = b.L[a];
        b.Lf[a] = (float)b.L[a];
    }
    b.ap = b.ar = 1.0;
    bool ok = true;
    if(P.precision != MTG_PREC_REFERENCE) {
        for(int a = 0; a < 3; a++) b.Lb[a] = b.L[a];
        ok = baro_box_fields(P, b);
    }
    *out = b;
    return ok;
}

// Output record of the last output step: U, K, T, P, V.  For a batch the per-replica records go
// to h_rrec and the returned record is the ensemble's: sums of U, K and V, T = 2 K / 3N over all
// atoms, P the mean of the replicas' pressures.
int read_records(mtg_ctx* c, double* rec) {
    if(!c->P.nrep) {
        CUDA_TRY(c, copy_now(c, rec, c->d.rec, sizeof(double) * 8, cudaMemcpyDeviceToHost));
        return MTG_OK;
    }
    const int nr = c->P.nrep;
    c->h_rrec.resize((size_t)nr * 8);
    CUDA_TRY(c, copy_now(c, c->h_rrec.data(), c->d.rrec, sizeof(double) * 8 * nr, cudaMemcpyDeviceToHost));
    for(int q = 0; q < 8; q++) rec[q] = 0.0;
    for(int r = 0; r < nr; r++) {
        const double* x = &c->h_rrec[(size_t)8 * r];
        rec[0] += x[0];
        rec[1] += x[1];
        rec[3] += x[3] / nr;
        rec[4] += x[4];
    }
    rec[2] = 2.0 * rec[1] / (3.0 * double(c->P.n));
    return MTG_OK;
}

// Applies the pending c2 to the device momenta and rewinds the thermostat (and, under NPT, the
// barostat) to the state after the last completed step (end of a run).
int settle_state(mtg_ctx* c) {
    // the kernels advance the double-float mirrors (mixed) and scale momenta lazily: bring the FP64
    // masters, the chains and the barostat to the completed step, on the device
    launch_settle(c->d, c->P, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    return MTG_OK;
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

int mtg_version(void) { return MTG_ABI_VERSION; }

int mtg_device_name(int device, char* buf, int buflen) {
    cudaDeviceProp prop;
    if(cudaGetDeviceProperties(&prop, device) != cudaSuccess) return MTG_E_CUDA;
    if(buf && buflen > 0) {
        std::snprintf(buf, (size_t)buflen, "%s (sm_%d%d, %d SMs)", prop.name, prop.major, prop.minor, prop.multiProcessorCount);
    }
    return MTG_OK;
}

int mtg_term_profile(const mtg_term* term, float x0, float x1, int npts, float* out) {
    if(!term || !out || npts < 2) return MTG_E_INVALID;
    const int k = term->kind;
    if(k >= MTG_NB_LJ && k <= MTG_NB_LJBUCK) return profile_nonbonded(k, term->p, x0, x1, npts, out);
    if(k >= MTG_BOND_HARM && k <= MTG_BOND_LJC) return profile_bond(k, term->p, x0, x1, npts, out);
    if(k >= MTG_ANGLE_HARM && k <= MTG_ANGLE_CLASS2) return profile_angle(k, term->p, x0, x1, npts, out);
    if(k >= MTG_DIH_HARM && k <= MTG_DIH_FOURIER4T) return profile_dihedral(k, term->p, x0, x1, npts, out);
    return MTG_E_UNSUPPORTED;
}

const char* mtg_last_error(const mtg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

void mtg_destroy(mtg_ctx* ctx) { delete ctx; }

static int create_impl(const mtg_system_desc* sys, const mtg_config_desc* cfg, const BatchSpec* bs, mtg_ctx** out) {
    g_create_error.clear();
    (void)cudaGetLastError();
    if(!sys || !cfg || !out) return fail(nullptr, MTG_E_INVALID, "null argument");
    *out = nullptr;
    const int n = sys->n_atoms, T = sys->n_types;
    if(n <= 0) return fail(nullptr, MTG_E_INVALID, "n_atoms must be positive");
    if(n > (int)kIdxMask) return fail(nullptr, MTG_E_INVALID, "too many atoms for 29-bit list indices");
    if(T <= 0 || !sys->type || !sys->r || !sys->mass || !sys->charge || !sys->nb_count)
        return fail(nullptr, MTG_E_INVALID, "missing atom arrays or non-bonded counts");
    for(int a = 0; a < 3; a++)
        if(!(sys->box[a] > 0.0) || !std::isfinite(sys->box[a])) return fail(nullptr, MTG_E_INVALID, "box widths must be positive");
    if(!finite_all(sys->r, (size_t)3 * n) || (sys->p && !finite_all(sys->p, (size_t)3 * n)) ||
       !finite_all(sys->mass, n) || !finite_all(sys->charge, n))
        return fail(nullptr, MTG_E_NONFINITE, "non-finite positions, momenta, masses or charges");
    for(int i = 0; i < n; i++) {
        if(sys->type[i] < 0 || sys->type[i] >= T) return fail(nullptr, MTG_E_INVALID, "atom type out of range");
        if(!(sys->mass[i] > 0.0)) return fail(nullptr, MTG_E_INVALID, "masses must be positive");
    }
    if(cfg->precision < MTG_PREC_REFERENCE || cfg->precision > MTG_PREC_MIXED) return fail(nullptr, MTG_E_INVALID, "bad precision");
    if(cfg->coulomb < MTG_COULOMB_ALLPAIRS || cfg->coulomb > MTG_COULOMB_SHIFTED) return fail(nullptr, MTG_E_INVALID, "bad coulomb mode");
    if(cfg->lj_shift < 0 || cfg->lj_shift > 2) return fail(nullptr, MTG_E_INVALID, "lj_shift must be 0, 1 or 2");
    if(cfg->precision == MTG_PREC_REFERENCE && cfg->coulomb != MTG_COULOMB_ALLPAIRS)
        return fail(nullptr, MTG_E_INVALID, "the reference precision mode has all-pairs Coulomb only");
    if(cfg->ensemble == MTG_NPT && (cfg->pressure_nh_len < 1 || cfg->pressure_nh_len > MTG_MAX_NH_CHAIN ||
                                    cfg->pressure_respa < 1 || !(cfg->pressure_relax > 0.0)))
        return fail(nullptr, MTG_E_INVALID, "NPT needs 1 <= pressure_nh_len <= MTG_MAX_NH_CHAIN, pressure_respa >= 1, pressure_relax > 0");
    if(cfg->ensemble != MTG_NVT && cfg->ensemble != MTG_NVE && cfg->ensemble != MTG_NPT) return fail(nullptr, MTG_E_INVALID, "bad ensemble");
    if(bs && (cfg->precision == MTG_PREC_REFERENCE || cfg->ensemble == MTG_NPT))
        return fail(nullptr, MTG_E_UNSUPPORTED, "batches run in the fp64 or mixed precision mode, NVT or NVE");
    if(cfg->temperature_nh_len < 0 || cfg->temperature_nh_len > kMaxChain) return fail(nullptr, MTG_E_INVALID, "chain length out of range");
    if(cfg->ensemble == MTG_NVT && (cfg->temperature_nh_len < 1 || cfg->temperature_respa < 1 || !(cfg->temperature > 0.0) || !(cfg->temperature_relax > 0.0)))
        return fail(nullptr, MTG_E_INVALID, "NVT needs temperature > 0, relaxation > 0, chain length >= 1, RESPA >= 1");
    if(!(cfg->timestep > 0.0) || !(cfg->cutoff_radius > 0.0)) return fail(nullptr, MTG_E_INVALID, "timestep and cutoff must be positive");
    for(int q = 0; q < T * T; q++)
        if(sys->nb_count[q] < 0 || sys->nb_count[q] > kMaxFF) return fail(nullptr, MTG_E_INVALID, "nb_count out of range");
    if(cfg->precision != MTG_PREC_REFERENCE && cfg->coulomb == MTG_COULOMB_ALLPAIRS) {
        bool anyq = false;
        for(int i = 0; i < n; i++) anyq |= (sys->charge[i] != 0.0);
        if(anyq) return fail(nullptr, MTG_E_UNSUPPORTED, "all-pairs Coulomb is available in the reference precision mode; use cutoff Coulomb with fp64/mixed");
    }
    auto check_topo = [&](int cnt, const int* a, int w, int ntypes) -> bool {
        if(cnt < 0 || (cnt > 0 && !a)) return false;
        for(int j = 0; j < cnt; j++) {
            for(int q = 0; q < w - 1; q++)
                if(a[w * j + q] < 0 || a[w * j + q] >= n) return false;
            if(a[w * j + w - 1] >= ntypes) return false;
        }
        return true;
    };
    if(!check_topo(sys->n_bonds, sys->bonds, 3, sys->n_bond_types) || !check_topo(sys->n_angles, sys->angles, 4, sys->n_angle_types) ||
       !check_topo(sys->n_dihedrals, sys->dihedrals, 5, sys->n_dih_types))
        return fail(nullptr, MTG_E_INVALID, "bonded topology indices out of range");

    std::unique_ptr<mtg_ctx> c(new mtg_ctx());
    c->cfg = *cfg;
    c->device = cfg->device;
    if(cudaSetDevice(c->device) != cudaSuccess) return fail(nullptr, MTG_E_CUDA, "cudaSetDevice failed (no GPU?)");
    if(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(nullptr, MTG_E_CUDA, "stream creation failed");
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);

    // ---- parameters ----
    Params& P = c->P;
    P.n = n;
    P.T = T;
    for(int a = 0; a < 3; a++) {
        P.box[a] = sys->box[a];
        P.boxf[a] = (float)sys->box[a];
        P.fscale[a] = (float)(sys->box[a] / 4294967296.0);
        P.fconv[a] = 4294967296.0 / sys->box[a];
    }
    P.ensemble = cfg->ensemble;
    P.precision = cfg->precision;
    P.coulomb = cfg->coulomb;
    P.clip = cfg->clip_forces;
    P.dt = cfg->timestep / kConvt;
    P.kT = cfg->temperature / kConvT;
    P.tau = cfg->temperature_relax / kConvt;
    P.M = cfg->ensemble == MTG_NVE ? 0 : cfg->temperature_nh_len;
    P.nresp = cfg->temperature_respa;
    P.fcut = cfg->cutoff_force;
    P.lj_shift = cfg->lj_shift;
    P.wait_polls = 1 << 22;
    {
        const double w0 = 1.0 / (2.0 - std::cbrt(2.0));
        P.chain_stage[0] = w0 * P.dt / double(P.nresp > 0 ? P.nresp : 1);
        P.chain_stage[1] = (1.0 - 2.0 * w0) * P.dt / double(P.nresp > 0 ? P.nresp : 1);
    }
    if(P.ensemble == MTG_NPT) {
        // SimulationBox.cpp:58-76: NH_P_ shares T; W = kT tauP^2, P_ = pressure / Conv_press, V0 = Lx Ly Lz
        const double tauP = cfg->pressure_relax / kConvt;
        P.MP = cfg->pressure_nh_len;
        P.nrespP = cfg->pressure_respa;
        P.Pext = cfg->pressure / kConvPress;
        P.QP = P.kT * tauP * tauP;
        // the production modes give the barostat the MTK mass (N_f + 3) kT tauP^2 (N_f = 3N), so
        // that tauP is its period; the reference's mass kT tauP^2 makes the volume of a system of
        // N atoms oscillate about sqrt(3N) times faster
        P.W = P.precision == MTG_PREC_REFERENCE ? P.QP : 3.0 * (double(sys->n_atoms) + 1.0) * P.QP;
        P.V0 = sys->box[0] * sys->box[1] * sys->box[2];
        P.clip = 0;   // the NPT branch does not clip forces (VelVerlet.cpp:57-71)
    }
    P.rc = (float)cfg->cutoff_radius;
    P.shell = (float)cfg->neigh_shell;
    P.rcoul = (float)(cfg->coulomb_cutoff > 0.0 ? cfg->coulomb_cutoff : cfg->cutoff_radius);
    P.skin = (float)(cfg->list_skin > 0.0 ? cfg->list_skin : 0.0);
    P.scale12 = (float)cfg->scale12;
    P.scale13 = (float)cfg->scale13;
    P.scale14 = (float)cfg->scale14;
    P.scale1N = (float)cfg->scale1N;
    P.scale[0] = 1.0f;
    P.scale[1] = P.scale12;
    P.scale[2] = P.scale13;
    P.scale[3] = P.scale14;
    P.scale[4] = P.scale1N;
    P.nx = ref_cells(sys->box[0], cfg->cutoff_radius, cfg->neigh_shell);
    P.ny = ref_cells(sys->box[1], cfg->cutoff_radius, cfg->neigh_shell);
    P.nz = ref_cells(sys->box[2], cfg->cutoff_radius, cfg->neigh_shell);
    if(P.nx < 1 || P.ny < 1 || P.nz < 1) return fail(nullptr, MTG_E_INVALID, "box narrower than cutoff + shell: the reference cell list is empty");
    // production cell grid of one box: cell edge >= rlist, or one cell when fewer than 3 fit
    auto grid = [&](const double* box, int natoms, int* pn, double rcv, double rqv) -> int {
        const double rlist = std::max(rcv, P.coulomb != MTG_COULOMB_ALLPAIRS ? rqv : 0.0) + P.skin;
        for(int a = 0; a < 3; a++) {
            pn[a] = (int)std::floor(box[a] / rlist);
            if(pn[a] < 3) pn[a] = 1;   // small box: scan every atom once (no duplicated images)
        }
        // keep the grid modest: at most ~ n/2 cells
        while((long long)pn[0] * pn[1] * pn[2] > std::max(27, natoms / 2)) {
            for(int a = 0; a < 3; a++) pn[a] = std::max(3, pn[a] - 1);
            if(pn[0] == 3 && pn[1] == 3 && pn[2] == 3) break;
        }
        if(P.precision != MTG_PREC_REFERENCE) {
            const double half = 0.5 * std::min(box[0], std::min(box[1], box[2]));
            if(rlist > half && (pn[0] > 1 || pn[1] > 1 || pn[2] > 1))
                return fail(nullptr, MTG_E_INVALID, "cutoff + skin exceeds half the box");
            if(std::max(rcv, rqv) >= half)
                return fail(nullptr, MTG_E_INVALID, "cutoff must be below half the box (minimum image)");
        }
        return MTG_OK;
    };
    std::vector<RepDev> reps;
    {
        int pn[3];
        int grc = bs ? 0 : grid(sys->box, n, pn, P.rc, P.rcoul);
        if(grc) return grc;
        if(bs) pn[0] = pn[1] = pn[2] = 1;   // unused: every replica has its own grid
        P.pnx = pn[0];
        P.pny = pn[1];
        P.pnz = pn[2];
    }
    c->ncell_ref = P.nx * P.ny * P.nz;
    c->ncell_prod = P.pnx * P.pny * P.pnz;
    c->nblocks_red = reduction_blocks(n);
    if(bs) {
        // replicas: contiguous atom ranges, whole 256-atom blocks each, own cell grid and box
        const int nr = bs->nrep;
        reps.resize(nr);
        int cb = 0, bb = 0;
        for(int r = 0; r < nr; r++) {
            RepDev& R = reps[r];
            R.off = bs->off[r];
            R.n = bs->n[r];
            R.bbase = bb;
            R.nb = reduction_blocks(R.n);
            bb += R.nb;
            for(int a = 0; a < 3; a++) {
                R.box[a] = bs->box[3 * r + a];
                R.fconv[a] = 4294967296.0 / R.box[a];
                R.fscale[a] = (float)(R.box[a] / 4294967296.0);
            }
            R.rc = bs->cutoff.empty() ? P.rc : (float)bs->cutoff[r];
            R.rcoul = bs->cutoff.empty() ? P.rcoul : (float)bs->cutoff[r];
            R.skin = P.skin;
            R.kT = bs->temperature[r] / kConvT;
            int pn[3];
            int grc = grid(R.box, R.n, pn, R.rc, R.rcoul);
            if(grc) return fail(nullptr, grc, "replica " + std::to_string(r) + ": " + g_create_error);
            R.cbase = cb;
            R.pnx = pn[0];
            R.pny = pn[1];
            R.pnz = pn[2];
            cb += pn[0] * pn[1] * pn[2];
        }
        P.nrep = nr;
        P.ncell_total = cb;
        P.nblk_total = bb;
        c->ncell_prod = cb;
        c->nblocks_red = bb;
        c->rep_off = bs->off;
        c->h_rep_box = bs->box;
    }

    // ---- tables ----
    const size_t TT = (size_t)T * T;
    std::vector<float> nb_tab(TT * kMaxFF * kNpts * 3, 0.0f);
    std::vector<int> nb_kind(TT * kMaxFF, 0);
    std::vector<double> nb_coef(TT * kMaxFF * 4, 0.0);
    std::vector<double> nb_fs(TT * kMaxFF, 0.0);
    std::vector<float> nb_coeff(TT * kMaxFF * 4, 0.0f);
    const float rcf = (float)cfg->cutoff_radius;
    for(size_t q = 0; q < TT; q++) {
        for(int ff = 0; ff < sys->nb_count[q]; ff++) {
            const size_t idx = q * kMaxFF + ff;
            const mtg_term& t = sys->nb_terms[idx];
            nb_kind[idx] = t.kind;
            if(sys->nb_tables) {
                std::memcpy(&nb_tab[idx * kNpts * 3], sys->nb_tables + idx * kNpts * 3, sizeof(float) * kNpts * 3);
            } else if(profile_nonbonded(t.kind, t.p, 0.01f, rcf, kNpts, &nb_tab[idx * kNpts * 3]) != MTG_OK) {
                return fail(nullptr, MTG_E_UNSUPPORTED, "non-bonded kind needs tables (LJBuck or unknown)");
            }
            // analytic coefficients (production modes)
            double* co = &nb_coef[idx * 4];
            if(t.kind == MTG_NB_LJ || t.kind == MTG_NB_LJ1208) {
                const double s2 = t.p[1] * t.p[1], s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s12 = s6 * s6;
                co[0] = 4.0 * t.p[0] * s12;
                co[1] = 4.0 * t.p[0] * t.p[2] * (t.kind == MTG_NB_LJ ? s6 : s8);
                // per-term cutoff^2 (0: the global cutoff applies), energy shift and cutoff force
                co[2] = t.p[3] > 0.0 ? t.p[3] * t.p[3] : 0.0;
                lj_shift_terms(t, co, cfg->cutoff_radius, cfg->lj_shift, &co[3], &nb_fs[idx]);
            } else if(t.kind == MTG_NB_BUCK) {
                co[0] = t.p[0];
                co[1] = (t.p[1] == 0.0) ? 1E-10 : 1.0 / t.p[1];
                co[2] = t.p[2];
            } else {
                nb_kind[idx] = 99;   // interpolate the table
            }
            for(int w = 0; w < 4; w++) nb_coeff[idx * 4 + w] = (float)co[w];
        }
    }
    auto bonded_tables = [&](int ntypes, const mtg_term* terms, const float* given, float x0, float x1,
                             int (*gen)(int, const double*, float, float, int, float*), std::vector<float>& tab,
                             std::vector<int>& kinds, std::vector<double>& par) -> int {
        tab.assign((size_t)std::max(ntypes, 1) * kNpts * 3, 0.0f);
        kinds.assign(std::max(ntypes, 1), 0);
        par.assign((size_t)std::max(ntypes, 1) * 4, 0.0);
        for(int t = 0; t < ntypes; t++) {
            kinds[t] = terms ? terms[t].kind : 99;
            if(terms) for(int w = 0; w < 4; w++) par[4 * t + w] = terms[t].p[w];
            if(given) std::memcpy(&tab[(size_t)t * kNpts * 3], given + (size_t)t * kNpts * 3, sizeof(float) * kNpts * 3);
            else if(!terms || gen(terms[t].kind, terms[t].p, x0, x1, kNpts, &tab[(size_t)t * kNpts * 3]) != MTG_OK)
                return MTG_E_UNSUPPORTED;
        }
        return MTG_OK;
    };
    std::vector<float> btab, atab, dtab;
    std::vector<int> bkind, akind, dkind;
    std::vector<double> bpar, apar, dpar;
    const float two_pi = float(2.0 * M_PI);
    if(bonded_tables(sys->n_bond_types, sys->bond_terms, sys->bond_tables, 0.01f, rcf, profile_bond, btab, bkind, bpar) ||
       bonded_tables(sys->n_angle_types, sys->angle_terms, sys->angle_tables, 0.0f, two_pi, profile_angle, atab, akind, apar) ||
       bonded_tables(sys->n_dih_types, sys->dih_terms, sys->dih_tables, 0.0f, two_pi, profile_dihedral, dtab, dkind, dpar))
        return fail(nullptr, MTG_E_UNSUPPORTED, "bonded kind needs tables (Class2 or unknown)");

    // ---- per-atom data ----
    std::vector<float> qf(n);
    std::vector<int> mol(n), mob(n), type(sys->type, sys->type + n);
    std::vector<float> invm(n);
    for(int i = 0; i < n; i++) {
        qf[i] = (float)sys->charge[i];
        mol[i] = sys->mol ? sys->mol[i] : -1;
        mob[i] = sys->mobile ? (sys->mobile[i] != 0) : 1;
        invm[i] = (float)(1.0 / sys->mass[i]);
    }
    c->h_mass.assign(sys->mass, sys->mass + n);
    c->h_mobile.resize(n);
    for(int i = 0; i < n; i++) c->h_mobile[i] = (uint8_t)mob[i];
    c->h_cfg = *cfg;
    c->h_type = type;
    c->h_nb_terms.assign(sys->nb_terms, sys->nb_terms + TT * kMaxFF);
    c->h_nb_count.assign(sys->nb_count, sys->nb_count + TT);
    c->h_nb_coef = nb_coef;
    c->h_nb_fs = nb_fs;
    c->h_charge.assign(sys->charge, sys->charge + n);
    c->has_tables = sys->nb_tables || sys->bond_tables || sys->angle_tables || sys->dih_tables;
    for(int k : nb_kind) c->has_tables |= (k == 99);
    for(int k : bkind) c->has_tables |= (k == 99 || k == MTG_BOND_LJC);
    for(int k : akind) c->has_tables |= (k == 99 || k == MTG_ANGLE_CLASS2);
    AtomLists L = build_atom_lists(n, sys->n_bonds, sys->bonds, sys->n_angles, sys->angles, sys->n_dihedrals, sys->dihedrals);

    DevSys& d = c->d;
    d.n = n;
    d.T = T;
    std::vector<double> p0((size_t)3 * n, 0.0);
    if(sys->p) std::memcpy(p0.data(), sys->p, sizeof(double) * 3 * n);
    for(int i = 0; i < n; i++)
        if(!mob[i]) p0[3 * i] = p0[3 * i + 1] = p0[3 * i + 2] = 0.0;   // SimulationBox.cpp:117-122
    int rc = 0;
    {
        mtg_ctx* C = c.get();
        rc = rc || upload(C, &d.r, sys->r, (size_t)3 * n);
        rc = rc || upload(C, &d.p, p0.data(), (size_t)3 * n);
        rc = rc || dalloc(C, &d.F, (size_t)3 * n);
        rc = rc || dalloc(C, &d.U, (size_t)n);
        if(P.precision != MTG_PREC_REFERENCE) rc = rc || dalloc(C, &d.W, (size_t)n);
        rc = rc || upload(C, &d.m, sys->mass, (size_t)n);
        rc = rc || upload(C, &d.qd, sys->charge, (size_t)n);
        rc = rc || upload(C, &d.qf, qf.data(), (size_t)n);
        rc = rc || upload(C, &d.type, type.data(), (size_t)n);
        rc = rc || upload(C, &d.mol, mol.data(), (size_t)n);
        rc = rc || upload(C, &d.mobile, mob.data(), (size_t)n);
        float* f;
        int* ip;
        double* dp;
        rc = rc || upload(C, &f, nb_tab.data(), nb_tab.size()); d.nb_tab = f;
        rc = rc || upload(C, &ip, sys->nb_count, TT); d.nb_cnt = ip;
        rc = rc || upload(C, &f, btab.data(), btab.size()); d.bond_tab = f;
        rc = rc || upload(C, &f, atab.data(), atab.size()); d.angle_tab = f;
        rc = rc || upload(C, &f, dtab.data(), dtab.size()); d.dih_tab = f;
        rc = rc || upload(C, &ip, nb_kind.data(), nb_kind.size()); d.nb_kind = ip;
        rc = rc || upload(C, &dp, nb_coef.data(), nb_coef.size()); d.nb_par = dp;
        rc = rc || upload(C, &f, nb_coeff.data(), nb_coeff.size()); d.nb_parf = f;
        {
            std::vector<float> fsf(nb_fs.begin(), nb_fs.end());
            rc = rc || upload(C, &dp, nb_fs.data(), nb_fs.size()); d.nb_fs = dp;
            rc = rc || upload(C, &f, fsf.data(), fsf.size()); d.nb_fsf = f;
            const std::vector<float> pcut = pair_cuts(c.get(), -1, -1);
            rc = rc || upload(C, &f, pcut.data(), pcut.size()); d.pair_cut = f;
            P.qon = charges_on(c.get());
            P.qany = any_charge(c.get());
        }
        // angle parameters on the device: (k, theta0 in radians, toRad, 0)
        for(size_t t = 0; t < akind.size(); t++) apar[4 * t + 1] = apar[4 * t + 1] * apar[4 * t + 2];
        c->h_bond_par = bpar;
        c->h_angle_par = apar;
        c->h_dih_par = dpar;
        c->h_bond_kind = bkind;
        c->h_angle_kind = akind;
        c->h_dih_kind = dkind;
        std::vector<float> bparf(bpar.begin(), bpar.end()), aparf(apar.begin(), apar.end()), dparf(dpar.begin(), dpar.end());
        rc = rc || upload(C, &ip, bkind.data(), bkind.size()); d.bond_kind = ip;
        rc = rc || upload(C, &dp, bpar.data(), bpar.size()); d.bond_par = dp;
        rc = rc || upload(C, &f, bparf.data(), bparf.size()); d.bond_parf = f;
        rc = rc || upload(C, &ip, akind.data(), akind.size()); d.angle_kind = ip;
        rc = rc || upload(C, &dp, apar.data(), apar.size()); d.angle_par = dp;
        rc = rc || upload(C, &f, aparf.data(), aparf.size()); d.angle_parf = f;
        rc = rc || upload(C, &ip, dkind.data(), dkind.size()); d.dih_kind = ip;
        rc = rc || upload(C, &dp, dpar.data(), dpar.size()); d.dih_par = dp;
        rc = rc || upload(C, &f, dparf.data(), dparf.size()); d.dih_parf = f;
        auto up = [&](const std::vector<int>& v) -> const int* {
            int* q = nullptr;
            rc = rc || upload(C, &q, v.data(), v.size());
            return q;
        };
        d.bptr = up(L.bptr); d.bj = up(L.bj); d.bt = up(L.bt);
        d.aptr = up(L.aptr); d.ai = up(L.ai); d.aj = up(L.aj); d.at = up(L.at); d.acen = up(L.acen);
        d.dptr = up(L.dptr); d.di = up(L.di); d.dj = up(L.dj); d.dl = up(L.dl); d.dt = up(L.dt); d.dcen = up(L.dcen);
        {
            std::vector<int> loc(n, 0);
            for(int k = 0; k < n; k++) {
                const int mk = mol[k];
                bool ok = mk >= 0;
                for(int e = L.bptr[k]; ok && e < L.bptr[k + 1]; e++) ok = mol[L.bj[e]] == mk;
                for(int e = L.aptr[k]; ok && e < L.aptr[k + 1]; e++) ok = L.acen[e] || mol[L.aj[e]] == mk;
                for(int e = L.dptr[k]; ok && e < L.dptr[k + 1]; e++) ok = L.dcen[e] || mol[L.dl[e]] == mk;
                loc[k] = ok ? 1 : 0;
            }
            d.excl_local = up(loc);
        }
        rc = rc || dalloc(C, &d.atom_cell, (size_t)3 * n);
        rc = rc || dalloc(C, &d.cell_first, (size_t)c->ncell_ref);
        rc = rc || dalloc(C, &d.cell_count, (size_t)c->ncell_ref);
        rc = rc || dalloc(C, &d.cell_cursor, (size_t)c->ncell_ref);
        rc = rc || dalloc(C, &d.cell_list, (size_t)n);
        rc = rc || dalloc(C, &d.nbr_count, (size_t)n);
        rc = rc || dalloc(C, &d.nbr_count_nb, (size_t)n);
        {
            // the reference-precision gather takes atoms grouped by type, so that the lanes of a
            // warp meet the same non-bonded terms (each atom's sums keep their own order)
            std::vector<int> order(n);
            for(int i = 0; i < n; i++) order[i] = i;
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return type[a] < type[b]; });
            rc = rc || upload(C, &d.force_order, order.data(), order.size());
        }
        rc = rc || dalloc(C, &d.pcell_of, (size_t)n);
        rc = rc || dalloc(C, &d.pcell_first, (size_t)c->ncell_prod);
        rc = rc || dalloc(C, &d.pcell_count, (size_t)c->ncell_prod);
        rc = rc || dalloc(C, &d.pcell_cursor, (size_t)c->ncell_prod);
        {
            // slot order starts as the identity; every list build replaces it with cell order
            std::vector<int> ident(n);
            for(int i = 0; i < n; i++) ident[i] = i;
            int* q = nullptr;
            rc = rc || upload(C, &q, ident.data(), ident.size());
            d.pcell_list = q;
            q = nullptr;
            rc = rc || upload(C, &q, ident.data(), ident.size());
            d.slot_of = q;
        }
        rc = rc || dalloc(C, &d.vcount, (size_t)n);
        rc = rc || dalloc(C, &d.vsr, (size_t)n);
        {
            std::vector<MixConst> mk;
            if(bs)
                for(const RepDev& R : reps) mk.push_back(mix_const_for(P, R.box, R.fconv, R.skin));
            else
                mk.push_back(mix_const_for(P, P.box, P.fconv, P.skin));
            MixConst* q = nullptr;
            rc = rc || upload(C, &q, mk.data(), mk.size());
            d.mixk = q;
        }
        rc = rc || dalloc(C, &d.r_build, (size_t)3 * n);
        rc = rc || dalloc(C, &d.rb4, (size_t)n);
        rc = rc || dalloc(C, &d.rb4s, (size_t)n);
        rc = rc || dalloc(C, &d.hi, (size_t)n);
        rc = rc || dalloc(C, &d.lo, (size_t)n);
        rc = rc || dalloc(C, &d.pq, (size_t)n);
        rc = rc || dalloc(C, &d.pqs, (size_t)n);
        rc = rc || dalloc(C, &d.ph, (size_t)n);
        rc = rc || dalloc(C, &d.pl, (size_t)n);
        {
            // per-type charge table, used when every atom of a type carries the same charge
            std::vector<float> qt(std::max(T, 1), 0.0f);
            std::vector<int> seen(std::max(T, 1), 0);
            bool uniform = T <= 8;
            for(int i = 0; i < n && uniform; i++) {
                const float q = (float)sys->charge[i];
                const int t = sys->type[i];
                if(!seen[t]) { seen[t] = 1; qt[t] = q; }
                else if(qt[t] != q) uniform = false;
            }
            P.qtype = uniform ? 1 : 0;
            float* qtd = nullptr;
            rc = rc || upload(C, &qtd, qt.data(), qt.size());
            d.qtype = qtd;
        }
        rc = rc || dalloc(C, &d.Fx, (size_t)n);
        rc = rc || dalloc(C, &d.Fy, (size_t)n);
        rc = rc || dalloc(C, &d.Fz, (size_t)n);
        rc = rc || upload(C, &d.inv_m, invm.data(), (size_t)n);
        rc = rc || dalloc(C, &d.partial, (size_t)c->nblocks_red * 4);
        rc = rc || dalloc(C, &d.sc, 1);
        rc = rc || dalloc(C, &d.th, 1);
        rc = rc || dalloc(C, &d.th_saved, 1);
        rc = rc || dalloc(C, &d.rec, 8);
        rc = rc || dalloc(C, &d.baro, 1);
        rc = rc || dalloc(C, &d.thp, 1);
        rc = rc || dalloc(C, &d.thp_saved, 1);
        if(bs) {
            const int nr = bs->nrep;
            std::vector<int> rep_of(n), blk_rep(P.nblk_total);
            for(int r = 0; r < nr; r++) {
                for(int i = reps[r].off; i < reps[r].off + reps[r].n; i++) rep_of[i] = r;
                for(int b = reps[r].bbase; b < reps[r].bbase + reps[r].nb; b++) blk_rep[b] = r;
            }
            int* ip2 = nullptr;
            rc = rc || upload(C, &ip2, rep_of.data(), rep_of.size()); d.rep_of = ip2;
            rc = rc || upload(C, &ip2, blk_rep.data(), blk_rep.size()); d.blk_rep = ip2;
            RepDev* rp = nullptr;
            rc = rc || upload(C, &rp, reps.data(), reps.size()); d.reps = rp;
            // chains: Q0 = 3 N_r kT_r tau^2, Qj = kT_r tau^2 (NHChain.cpp:115-124), per replica
            std::vector<ThermoDev> ths(nr);
            std::vector<StepScalars> rs(nr);
            for(int r = 0; r < nr; r++) {
                ThermoDev& th = ths[r];
                for(int j = 0; j < kMaxChain; j++) th.Q[j] = 1.0;
                if(P.M > 0) {
                    th.Q[0] = double(3 * reps[r].n) * reps[r].kT * P.tau * P.tau;
                    for(int j = 1; j < P.M; j++) th.Q[j] = reps[r].kT * P.tau * P.tau;
                }
                for(int j = 0; j < kMaxChain; j++) th.iQ[j] = 1.0 / th.Q[j];
                rs[r].S = 1.0;
                rs[r].c2 = 1.0;
            }
            rc = rc || upload(C, &d.ths, ths.data(), ths.size());
            rc = rc || upload(C, &d.ths_saved, ths.data(), ths.size());
            rc = rc || upload(C, &d.rsc, rs.data(), rs.size());
            rc = rc || dalloc(C, &d.rrec, (size_t)8 * nr);
        }
    }
    if(rc) return fail(nullptr, rc, c->err);
    // thermostat masses (NHChain.cpp:115-124): Q0 = dim N kT tau^2, Qj = kT tau^2
    {
        ThermoDev th{};
        for(int j = 0; j < kMaxChain; j++) th.Q[j] = 1.0;
        if(P.M > 0) {
            th.Q[0] = double(3 * n) * P.kT * P.tau * P.tau;
            for(int j = 1; j < P.M; j++) th.Q[j] = P.kT * P.tau * P.tau;
        }
        for(int j = 0; j < kMaxChain; j++) th.iQ[j] = 1.0 / th.Q[j];
        copy_now(c.get(), d.th, &th, sizeof(th), cudaMemcpyHostToDevice);
        copy_now(c.get(), d.th_saved, &th, sizeof(th), cudaMemcpyHostToDevice);
        StepScalars s{};
        s.S = 1.0;
        s.c2 = 1.0;
        copy_now(c.get(), d.sc, &s, sizeof(s), cudaMemcpyHostToDevice);
        // barostat chain: prepareArrays(1, 1) gives Q0 = kT tauP^2 as well (NHChain.cpp:115-124)
        ThermoDev tp{};
        for(int j = 0; j < kMaxChain; j++) tp.Q[j] = 1.0;
        if(P.ensemble == MTG_NPT)
            for(int j = 0; j < P.MP; j++) tp.Q[j] = P.QP;
        for(int j = 0; j < kMaxChain; j++) tp.iQ[j] = 1.0 / tp.Q[j];
        copy_now(c.get(), d.thp, &tp, sizeof(tp), cudaMemcpyHostToDevice);
        copy_now(c.get(), d.thp_saved, &tp, sizeof(tp), cudaMemcpyHostToDevice);
        BaroDev b{};
        baro_at(P, 0.0, 0.0, &b);
        copy_now(c.get(), d.baro, &b, sizeof(b), cudaMemcpyHostToDevice);
    }
    // list capacities: start from a density estimate, grown on demand
    {
        // density of the system, or of the densest replica of a batch (the merged box is not one)
        const double V = sys->box[0] * sys->box[1] * sys->box[2];
        double rho = bs ? 0.0 : n / V;
        for(const RepDev& R : reps) rho = std::max(rho, R.n / (R.box[0] * R.box[1] * R.box[2]));
        const double rc3 = std::pow(cfg->cutoff_radius, 3.0);
        // the reference list is used every step only in reference mode; elsewhere (parity hooks)
        // it starts small and grows on demand
        int est = P.precision == MTG_PREC_REFERENCE ? (int)(1.3 * rho * 4.18879 * rc3) + 32 : 16;
        double rl = std::max((double)P.rc, P.coulomb != MTG_COULOMB_ALLPAIRS ? (double)P.rcoul : 0.0) + P.skin;
        int vest = (int)(1.2 * rho * 4.18879 * rl * rl * rl) + 32;
        if(cfg->initial_max_neighbours > 0) {
            // the caller's first capacity (the reference starts at 10): lists grow on overflow
            rc = grow_neighbors(c.get(), std::max(0, cfg->initial_max_neighbours - 10));
            if(rc) return fail(nullptr, rc, c->err);
            rc = grow_vlist(c.get(), cfg->initial_max_neighbours, true);
        } else {
            rc = grow_neighbors(c.get(), std::min(est, n));
            if(rc) return fail(nullptr, rc, c->err);
            rc = grow_vlist(c.get(), std::min(vest, n));
        }
        if(rc) return fail(nullptr, rc, c->err);
    }
    if(is_mixed(c.get())) launch_prod_sync(d, P, kSyncFromMaster, c->stream);
    // snapshot set for chunk rollback
    {
        mtg_ctx* C = c.get();
        rc = rc || add_snap(C, d.r, sizeof(double) * 3 * n);
        rc = rc || add_snap(C, d.p, sizeof(double) * 3 * n);
        rc = rc || add_snap(C, d.F, sizeof(double) * 3 * n);
        rc = rc || add_snap(C, d.U, sizeof(double) * n);
        rc = rc || add_snap(C, d.th, sizeof(ThermoDev));
        rc = rc || add_snap(C, d.th_saved, sizeof(ThermoDev));
        rc = rc || add_snap(C, d.sc, sizeof(StepScalars));
        if(bs) {
            rc = rc || add_snap(C, d.rsc, sizeof(StepScalars) * bs->nrep);
            rc = rc || add_snap(C, d.ths, sizeof(ThermoDev) * bs->nrep);
            rc = rc || add_snap(C, d.ths_saved, sizeof(ThermoDev) * bs->nrep);
        }
        if(P.ensemble == MTG_NPT) {
            rc = rc || add_snap(C, d.baro, sizeof(BaroDev));
            rc = rc || add_snap(C, d.thp, sizeof(ThermoDev));
            rc = rc || add_snap(C, d.thp_saved, sizeof(ThermoDev));
            if(P.precision != MTG_PREC_REFERENCE) rc = rc || add_snap(C, d.W, sizeof(double) * n);
        }
        if(is_mixed(C)) {
            rc = rc || add_snap(C, d.hi, sizeof(float4) * n);
            rc = rc || add_snap(C, d.lo, sizeof(float4) * n);
            rc = rc || add_snap(C, d.pq, sizeof(uint4) * n);
            rc = rc || add_snap(C, d.ph, sizeof(float4) * n);
            rc = rc || add_snap(C, d.pl, sizeof(float4) * n);
            rc = rc || add_snap(C, d.Fx, sizeof(long long) * n);
            rc = rc || add_snap(C, d.Fy, sizeof(long long) * n);
            rc = rc || add_snap(C, d.Fz, sizeof(long long) * n);
        }
        if(rc) return fail(nullptr, rc, c->err);
    }
    P.team = 32;
    rc = compute_forces_now(c.get(), true);
    if(rc) return fail(nullptr, rc, c->err);
    if(!is_reference(c.get())) {
        rc = autotune_force(c.get());
        if(rc) return fail(nullptr, rc, c->err);
    }
    if(cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(nullptr, MTG_E_CUDA, "initial force evaluation failed");
    *out = c.release();
    return MTG_OK;
}

int mtg_create(const mtg_system_desc* sys, const mtg_config_desc* cfg, mtg_ctx** out) {
    return create_impl(sys, cfg, nullptr, out);
}

int mtg_set_state(mtg_ctx* c, const double* r, const double* p, const mtg_thermo_state* th) {
    if(!c) return MTG_E_INVALID;
    const size_t n3 = (size_t)c->P.n * 3;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    if(r && !finite_all(r, n3)) return fail(c, MTG_E_NONFINITE, "non-finite positions");
    if(p && !finite_all(p, n3)) return fail(c, MTG_E_NONFINITE, "non-finite momenta");
    // stream-ordered uploads; the force evaluation below synchronises once (from pageable memory
    // the copy has left the caller's buffer when cudaMemcpyAsync returns)
    if(r) CUDA_TRY(c, cudaMemcpyAsync(c->d.r, r, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if(p) CUDA_TRY(c, cudaMemcpyAsync(c->d.p, p, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if(th && c->P.nrep) return fail(c, MTG_E_INVALID, "a batch sets chain states per replica (mtg_batch_set_thermo)");
    const bool box_changes = th && c->P.ensemble == MTG_NPT;
    if(th) {
        // chain and barostat values go to the device as kernel arguments (no synchronous copy)
        ChainSet cs{};
        cs.M = std::max(0, std::min<int>(th->M, kMaxChain));
        for(int j = 0; j < cs.M; j++) {
            cs.eta[j] = th->eta[j];
            cs.peta[j] = th->p_eta[j];
        }
        if(c->P.ensemble == MTG_NPT) {
            if(!std::isfinite(th->p_eps) || !std::isfinite(th->eps)) return fail(c, MTG_E_NONFINITE, "non-finite barostat state");
            cs.MP = std::max(0, std::min<int>(th->MP, kMaxChain));
            for(int j = 0; j < cs.MP; j++) {
                cs.etaP[j] = th->etaP[j];
                cs.petaP[j] = th->p_etaP[j];
            }
            if(!baro_at(c->P, th->p_eps, th->eps, &cs.baro, th->box))
                return fail(c, MTG_E_UNSUPPORTED, "the barostat state's box is narrower than twice the cutoff");
            cs.set_baro = 1;
        }
        launch_set_chains(c->d, cs, c->stream);
        CUDA_TRY(c, cudaGetLastError());
    }
    // mixed: the double-float mirrors and the box fractions, in the box just set
    if(is_mixed(c)) {
        if(r || p) launch_prod_sync(c->d, c->P, kSyncFromMaster, c->stream);
        else if(box_changes) launch_prod_sync(c->d, c->P, kSyncPositionsFromMaster, c->stream);
    }
    if(r || box_changes) return compute_forces_now(c, true, !box_changes);
    return MTG_OK;
}

int mtg_get_state(mtg_ctx* c, double* r, double* p, mtg_thermo_state* th) {
    if(!c) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    const size_t n3 = (size_t)c->P.n * 3;
    if(th && c->P.nrep) return fail(c, MTG_E_INVALID, "a batch reads chain states per replica (mtg_batch_get_thermo)");
    // settle_state has brought the FP64 masters up to date (mixed: from the double-float mirrors)
    if(r) CUDA_TRY(c, cudaMemcpyAsync(r, c->d.r, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if(p) CUDA_TRY(c, cudaMemcpyAsync(p, c->d.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    const bool npt = c->P.ensemble == MTG_NPT;
    if(th) {
        if(!c->pin_th) CUDA_TRY(c, cudaMallocHost((void**)&c->pin_th, sizeof(mtg_ctx::ThermoStage)));
        CUDA_TRY(c, cudaMemcpyAsync(&c->pin_th->th, c->d.th, sizeof(ThermoDev), cudaMemcpyDeviceToHost, c->stream));
        if(npt) {
            CUDA_TRY(c, cudaMemcpyAsync(&c->pin_th->thp, c->d.thp, sizeof(ThermoDev), cudaMemcpyDeviceToHost, c->stream));
            CUDA_TRY(c, cudaMemcpyAsync(&c->pin_th->baro, c->d.baro, sizeof(BaroDev), cudaMemcpyDeviceToHost, c->stream));
        }
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if(th) {
        const ThermoDev& t = c->pin_th->th;
        std::memset(th, 0, sizeof(*th));
        th->M = c->P.M;
        for(int j = 0; j < c->P.M; j++) {
            th->eta[j] = t.eta[j];
            th->p_eta[j] = t.peta[j];
        }
        for(int a = 0; a < 3; a++) th->box[a] = c->P.box[a];
        if(npt) {
            const ThermoDev& tp = c->pin_th->thp;
            const BaroDev& b = c->pin_th->baro;
            th->MP = c->P.MP;
            for(int j = 0; j < c->P.MP; j++) {
                th->etaP[j] = tp.eta[j];
                th->p_etaP[j] = tp.peta[j];
            }
            th->p_eps = b.p_eps;
            th->eps = b.eps;
            for(int a = 0; a < 3; a++) th->box[a] = b.L[a];
        }
    }
    return MTG_OK;
}

// Longest chunk of steps in one step graph (a run without output steps is cut into chunks of this
// length: each chunk is one graph launch, a snapshot for the overflow redo and one host check).
constexpr int kMaxChunk = 100;

int mtg_run(mtg_ctx* c, int nsteps, int out_stride, mtg_output_cb cb, void* user) {
    if(!c || nsteps < 0) return MTG_E_INVALID;
    if(nsteps == 0) return MTG_OK;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if(out_stride < 0) out_stride = 0;   // 0: no output steps
    c->stats = mtg_run_stats{};
    if(!c->team_retuned && !is_reference(c) && c->P.nrep == 0) {
        // the team size chosen at creation was timed on the starting configuration; re-time it
        // once on the one that runs (forces do not depend on it: integer sums)
        c->team_retuned = true;
        const int before = c->P.team;
        const int rc = autotune_force(c, true);
        if(rc) return rc;
        if(c->P.team != before) drop_graphs(c);   // captured graphs hold the old team size
    }
    cudaMemsetAsync(&c->d.sc->builds_run, 0, sizeof(int32_t), c->stream);
    // thermostat first half-step of step 0 from the current momenta
    launch_prologue(c->d, c->P, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    float total_ms = 0.0f;
    int t = 0;
    int gen_seen = c->generation;
    PendingOutput pend;       // the previous output step, delivered while the next chunk runs
    int nout = 0;
    int64_t last_done = -1;   // last step of the chunk before the one in flight
    while(t < nsteps) {
        // chunk: up to the next output step (t % out_stride == 0) inclusive, at most kMaxChunk steps
        int end = nsteps - 1;
        if(out_stride > 0) end = std::min(end, (t % out_stride == 0) ? t : (t / out_stride + 1) * out_stride);
        end = std::min(end, t + kMaxChunk - 1);
        const bool output = out_stride > 0 && end % out_stride == 0;
        const int steps = end - t + 1;
        int attempt = 0;
        for(;;) {
            if(c->generation != gen_seen) {
                drop_graphs(c);
                gen_seen = c->generation;
            }
            take_snapshot(c);
            clear_overflow(c);
            cudaGraphExec_t ge;
            int rc = get_graph(c, steps, output, choose_form(c, steps), &ge);
            if(rc) return rc;
            const int form = c->last_form;
            CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
            CUDA_TRY(c, cudaGraphLaunch(ge, c->stream));
            CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
            // the previous output step's callback runs on the host while this chunk runs
            if(pend.live) {
                bool stop = false;
                rc = deliver_output(c, pend, cb, user, &stop);
                if(rc) return rc;
                if(stop) {
                    // undo the chunk in flight: back to the state after the delivered step
                    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
                    restore_snapshot(c);
                    c->stats.steps = last_done + 1;
                    c->stats.device_ms = total_ms;
                    return settle_state(c);
                }
            }
            StepScalars s = read_scalars(c);
            CUDA_TRY(c, cudaGetLastError());
            if(s.overflow) {
                restore_snapshot(c);
                if(is_reference(c)) rc = grow_neighbors(c, s.needed);
                else {
                    rc = grow_vlist(c, s.needed);
                    cudaMemsetAsync(&c->d.sc->rebuild, 0xff, sizeof(int32_t), c->stream);
                }
                if(rc) return rc;
                if(++attempt > 32) return fail(c, MTG_E_OVERFLOW, "neighbour list did not converge");
                continue;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            total_ms += ms;
            record_form(c, form, steps, ms);
            if(s.timeout) return fail(c, MTG_E_TIMEOUT, "a bounded wait in the thermostat gave up");
            if(s.boxerr) return fail(c, MTG_E_UNSUPPORTED, "NPT: the box shrank until a cutoff reached half its width");
            if(s.nonfinite) return fail(c, MTG_E_NONFINITE, "non-finite kinetic energy or thermostat scale during the run");
            c->stats.list_builds = s.builds_run;
            if(output) {
                double rec[8];
                int rrc = read_records(c, rec);
                if(rrc) return rrc;
                if(!std::isfinite(rec[0]) || !std::isfinite(rec[1])) return fail(c, MTG_E_NONFINITE, "non-finite energy during the run");
                if(cb) {
                    int frc = queue_output(c, nout & 1, s.c2, pend);
                    if(frc) return frc;
                    pend.step = end;
                    std::memcpy(pend.rec, rec, sizeof rec);
                    nout++;
                }
            }
            break;
        }
        last_done = end;
        t = end + 1;
        c->stats.graph_steps = steps;
    }
    if(pend.live) {
        bool stop = false;
        int rc = deliver_output(c, pend, cb, user, &stop);
        if(rc) return rc;
    }
    c->stats.steps = nsteps;
    c->stats.device_ms = total_ms;
    // prologue + per-step kernels + the six build kernels of every production rebuild
    c->stats.kernel_launches = (int64_t)nsteps * kernels_per_step(c) + 1 + (is_reference(c) ? 0 : 6 * c->stats.list_builds);
    c->stats.force_team = c->P.team;
    c->stats.graph_form = is_reference(c) ? 0 : c->graph_form;
    return settle_state(c);
}

int mtg_compute_forces(mtg_ctx* c, double* F, double* Fpi, double* U) {
    if(!c) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    rc = compute_forces_now(c, true);
    if(rc) return rc;
    if(is_mixed(c)) launch_prod_forces_to_double(c->d, c->P, c->stream);
    const size_t n3 = (size_t)c->P.n * 3;
    if(F) CUDA_TRY(c, cudaMemcpyAsync(F, c->d.F, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if(Fpi) CUDA_TRY(c, cudaMemcpyAsync(Fpi, c->d.F, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if(U) CUDA_TRY(c, cudaMemcpyAsync(U, c->d.U, (size_t)c->P.n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MTG_OK;
}

int mtg_get_cells(mtg_ctx* c, int32_t* dims, int32_t* ixyz, int32_t* cell_first, int32_t* cell_count, int32_t ncells,
                  int32_t* cell_list) {
    if(!c) return MTG_E_INVALID;
    if(c->P.nrep) return fail(c, MTG_E_UNSUPPORTED, "the reference cell list is not built for batches");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if(dims) {
        dims[0] = c->P.nx;
        dims[1] = c->P.ny;
        dims[2] = c->P.nz;
    }
    if((cell_first || cell_count) && ncells < c->ncell_ref) return fail(c, MTG_E_INVALID, "cell arrays too small");
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncToMaster, c->stream);
    launch_ref_cells(c->d, c->P, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    const int n = c->P.n;
    if(ixyz) CUDA_TRY(c, cudaMemcpyAsync(ixyz, c->d.atom_cell, sizeof(int) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    if(cell_first) CUDA_TRY(c, cudaMemcpyAsync(cell_first, c->d.cell_first, sizeof(int) * c->ncell_ref, cudaMemcpyDeviceToHost, c->stream));
    if(cell_count) CUDA_TRY(c, cudaMemcpyAsync(cell_count, c->d.cell_count, sizeof(int) * c->ncell_ref, cudaMemcpyDeviceToHost, c->stream));
    if(cell_list) CUDA_TRY(c, cudaMemcpyAsync(cell_list, c->d.cell_list, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MTG_OK;
}

int mtg_get_neighbors(mtg_ctx* c, int32_t max_neigh, int32_t* count, int32_t* list, int32_t* needed) {
    if(!c) return MTG_E_INVALID;
    if(c->P.nrep) return fail(c, MTG_E_UNSUPPORTED, "the reference neighbour list is not built for batches");
    CUDA_TRY(c, cudaSetDevice(c->device));
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncToMaster, c->stream);
    for(int attempt = 0; attempt < 64; attempt++) {
        clear_overflow(c);
        launch_ref_cells(c->d, c->P, c->stream);
        launch_ref_neigh(c->d, c->P, c->stream);
        CUDA_TRY(c, cudaGetLastError());
        StepScalars s = read_scalars(c);
        if(!s.overflow) break;
        int rc = grow_neighbors(c, s.needed);
        if(rc) return rc;
    }
    const int n = c->P.n;
    std::vector<int> cnt(n);
    CUDA_TRY(c, copy_now(c, cnt.data(), c->d.nbr_count, sizeof(int) * n, cudaMemcpyDeviceToHost));
    int mx = 0;
    for(int v : cnt) mx = std::max(mx, v);
    if(needed) *needed = mx;
    if(count) std::memcpy(count, cnt.data(), sizeof(int) * n);
    if(list) {
        if(max_neigh < mx) return fail(c, MTG_E_INVALID, "max_neigh smaller than the longest list");
        std::vector<int> tmp((size_t)n * c->d.nbr_max);
        CUDA_TRY(c, copy_now(c, tmp.data(), c->d.nbr_list, tmp.size() * sizeof(int), cudaMemcpyDeviceToHost));
        for(int k = 0; k < n; k++)
            for(int e = 0; e < max_neigh; e++) list[(size_t)k * max_neigh + e] = e < cnt[k] ? tmp[(size_t)k * c->d.nbr_max + e] : -1;
    }
    return MTG_OK;
}

int mtg_optimize(mtg_ctx* c, double accuracy, int max_steps, int out_stride, mtg_output_cb cb, void* user) {
    // CMDLoop::runOptimization (MDLoop.cpp:143-173): F at the current positions, r += lr F,
    // U_{n+1} = U(F's positions), stop when |U_{n+1} - U_n| < accuracy after more than out_stride steps.
    if(!c || max_steps < 0) return MTG_E_INVALID;
    if(c->P.nrep) return fail(c, MTG_E_UNSUPPORTED, "gradient descent runs on single systems; relax replicas before batching");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    if(out_stride <= 0) out_stride = max_steps + 1;
    const double lr = c->cfg.opt_learning_rate;
    double U_n = 0.0;
    {
        rc = compute_forces_now(c, true);
        if(rc) return rc;
        std::vector<double> U(c->P.n);
        CUDA_TRY(c, copy_now(c, U.data(), c->d.U, sizeof(double) * c->P.n, cudaMemcpyDeviceToHost));
        for(double u : U) U_n += u;
    }
    c->stats = mtg_run_stats{};
    for(int i = 0; i < max_steps; i++) {
        // forces at the current positions (reference: lists rebuilt; production: rebuilt when due)
        for(int attempt = 0;; attempt++) {
            clear_overflow(c);
            if(is_reference(c)) {
                launch_ref_cells(c->d, c->P, c->stream);
                launch_ref_neigh(c->d, c->P, c->stream);
                launch_ref_force(c->d, c->P, c->stream);
            } else {
                launch_prod_build(c->d, c->P, false, c->stream);
                launch_prod_force(c->d, c->P, true, c->stream);
            }
            StepScalars s = read_scalars(c);
            CUDA_TRY(c, cudaGetLastError());
            if(!s.overflow) break;
            rc = is_reference(c) ? grow_neighbors(c, s.needed) : grow_vlist(c, s.needed);
            if(rc) return rc;
            if(!is_reference(c)) cudaMemsetAsync(&c->d.sc->rebuild, 0xff, sizeof(int32_t), c->stream);
            if(attempt > 32) return fail(c, MTG_E_OVERFLOW, "neighbour list did not converge");
        }
        launch_gd_step(c->d, c->P, lr, c->stream);
        double rec[8];
        CUDA_TRY(c, cudaMemcpyAsync(rec, c->d.rec, sizeof(rec), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if(!std::isfinite(rec[0])) return fail(c, MTG_E_NONFINITE, "non-finite energy during optimisation");
        const double U_np1 = rec[0];
        const double Udiff = std::fabs(U_np1 - U_n);
        U_n = U_np1;
        c->stats.steps = i + 1;
        if(cb && (i % out_stride) == 0) {
            rc = fetch_rp(c, 1.0);
            if(rc) return rc;
            mtg_output o{};
            o.step = i;
            o.U = rec[0];
            o.K = rec[1];
            o.T = rec[2];
            o.P = rec[3];
            o.V = rec[4];
            o.E = rec[0] + rec[1];
            o.r = c->h_r.data();
            o.p = c->h_p.data();
            if(cb(&o, user)) break;
        }
        if((Udiff < accuracy) && (i > out_stride)) break;
    }
    // forces at the final positions for the next run
    rc = compute_forces_now(c, true);
    return rc;
}

int mtg_profile_phases(mtg_ctx* c, int steps, double* phase_ms) {
    if(!c || steps <= 0 || !phase_ms) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    cudaEvent_t ev[6];
    for(auto& e : ev) CUDA_TRY(c, cudaEventCreate(&e));
    double acc[5] = {0, 0, 0, 0, 0};
    launch_prologue(c->d, c->P, c->stream);
    take_snapshot(c);
    clear_overflow(c);
    for(int s = 0; s < steps; s++) {
        cudaEventRecord(ev[0], c->stream);
        if(is_reference(c)) launch_ref_kick_drift(c->d, c->P, c->stream);
        else launch_prod_kick_drift(c->d, c->P, c->stream);
        cudaEventRecord(ev[1], c->stream);
        if(is_reference(c)) {
            launch_ref_cells(c->d, c->P, c->stream);
            launch_ref_neigh(c->d, c->P, c->stream);
        } else {
            launch_prod_build(c->d, c->P, false, c->stream);
        }
        cudaEventRecord(ev[2], c->stream);
        if(is_reference(c)) launch_ref_force(c->d, c->P, c->stream);
        else launch_prod_force(c->d, c->P, false, c->stream);
        cudaEventRecord(ev[3], c->stream);
        if(is_reference(c)) launch_ref_kick2(c->d, c->P, false, c->stream);
        else launch_prod_kick2(c->d, c->P, false, c->stream, kKick2Atoms);
        cudaEventRecord(ev[4], c->stream);
        if(!is_reference(c)) launch_prod_kick2(c->d, c->P, false, c->stream, kKick2StepEnd);
        cudaEventRecord(ev[5], c->stream);
        CUDA_TRY(c, cudaEventSynchronize(ev[5]));
        for(int q = 0; q < 5; q++) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
            acc[q] += ms;
        }
    }
    for(auto& e : ev) cudaEventDestroy(e);
    CUDA_TRY(c, cudaGetLastError());
    StepScalars sc = read_scalars(c);
    if(sc.overflow) {
        restore_snapshot(c);
        int rc = is_reference(c) ? grow_neighbors(c, sc.needed) : grow_vlist(c, sc.needed);
        if(rc) return rc;
        return fail(c, MTG_E_OVERFLOW, "list grew during profiling; state restored, call again");
    }
    for(int q = 0; q < 5; q++) phase_ms[q] = acc[q] / steps;
    return settle_state(c);
}

int mtg_draw_initial_state(const mtg_system_desc* sys, const mtg_config_desc* cfg, uint32_t seed, int32_t mode, double* p,
                           mtg_thermo_state* th) {
    g_create_error.clear();
    if(!sys || !cfg || !p || !th || sys->n_atoms <= 0 || !sys->mass)
        return fail(nullptr, MTG_E_INVALID, "mtg_draw_initial_state: null argument or no atoms");
    if(mode != MTG_INIT_REFERENCE && mode != MTG_INIT_MAXWELL)
        return fail(nullptr, MTG_E_INVALID, "mtg_draw_initial_state: unknown mode");
    const int rc = draw_initial_state(sys->n_atoms, sys->mass, sys->mobile, cfg, seed, mode, p, th);
    if(rc) return fail(nullptr, rc, "mtg_draw_initial_state: chain lengths must lie in 0 .. MTG_MAX_NH_CHAIN");
    return MTG_OK;
}

int mtg_init_state(mtg_ctx* c, uint32_t seed, int32_t mode) {
    if(!c) return MTG_E_INVALID;
    if(c->P.nrep) return fail(c, MTG_E_UNSUPPORTED, "a batch takes per-replica states (mtg_set_state, mtg_batch_set_thermo)");
    if(mode != MTG_INIT_REFERENCE && mode != MTG_INIT_MAXWELL) return fail(c, MTG_E_INVALID, "unknown initial-state mode");
    const int n = c->P.n;
    std::vector<double> p((size_t)3 * n);
    mtg_thermo_state th{};
    int rc = draw_initial_state(n, c->h_mass.data(), c->h_mobile.data(), &c->h_cfg, seed, mode, p.data(), &th);
    if(rc) return fail(c, rc, "initial state: chain lengths must lie in 0 .. MTG_MAX_NH_CHAIN");
    th.eps = 0.0;
    return mtg_set_state(c, nullptr, p.data(), &th);
}

int mtg_set_wait_limit(mtg_ctx* c, int32_t polls) {
    if(!c) return MTG_E_INVALID;
    if(polls < 0) return fail(c, MTG_E_INVALID, "wait limit must be non-negative");
    c->P.wait_polls = polls;
    drop_graphs(c);   // captured launches carry the parameters by value
    return MTG_OK;
}

int mtg_get_run_stats(mtg_ctx* c, mtg_run_stats* st) {
    if(!c || !st) return MTG_E_INVALID;
    *st = c->stats;
    return MTG_OK;
}

// ---------------------------------------------------------------------------------------------
// Batches of replicas
// ---------------------------------------------------------------------------------------------
int mtg_batch_create(const mtg_system_desc* const* systems, int32_t nrep, const mtg_config_desc* cfg,
                     const double* temperatures, const double* cutoffs, mtg_ctx** out) {
    g_create_error.clear();
    if(!systems || nrep < 1 || !cfg || !out) return fail(nullptr, MTG_E_INVALID, "null argument or no replicas");
    *out = nullptr;
    const mtg_system_desc* s0 = systems[0];
    if(!s0) return fail(nullptr, MTG_E_INVALID, "null replica");
    const int T = s0->n_types;
    if(T <= 0 || !s0->nb_count) return fail(nullptr, MTG_E_INVALID, "replica 0: missing types");
    auto same_terms = [](const mtg_term* a, const mtg_term* b, int cnt) -> bool {
        for(int q = 0; q < cnt; q++) {
            if(a[q].kind != b[q].kind) return false;
            for(int w = 0; w < 4; w++)
                if(a[q].p[w] != b[q].p[w]) return false;
        }
        return true;
    };
    long long N = 0;
    for(int r = 0; r < nrep; r++) {
        const mtg_system_desc* s = systems[r];
        if(!s || s->n_atoms <= 0 || !s->r || !s->mass || !s->charge || !s->type || !s->nb_count)
            return fail(nullptr, MTG_E_INVALID, "replica " + std::to_string(r) + ": missing atom arrays");
        if(s->n_types != T || s->n_bond_types != s0->n_bond_types || s->n_angle_types != s0->n_angle_types ||
           s->n_dih_types != s0->n_dih_types)
            return fail(nullptr, MTG_E_INVALID, "replica " + std::to_string(r) + ": replicas must share one force field");
        if(s->nb_tables || s->bond_tables || s->angle_tables || s->dih_tables)
            return fail(nullptr, MTG_E_UNSUPPORTED, "batches use the analytic terms (no tables)");
        for(int q = 0; q < T * T; q++) {
            if(s->nb_count[q] != s0->nb_count[q] || s->nb_count[q] < 0 || s->nb_count[q] > kMaxFF ||
               !same_terms(s->nb_terms + q * kMaxFF, s0->nb_terms + q * kMaxFF, s->nb_count[q]))
                return fail(nullptr, MTG_E_INVALID, "replica " + std::to_string(r) + ": replicas must share one force field");
        }
        if(!same_terms(s->bond_terms, s0->bond_terms, s0->n_bond_types) || !same_terms(s->angle_terms, s0->angle_terms, s0->n_angle_types) ||
           !same_terms(s->dih_terms, s0->dih_terms, s0->n_dih_types))
            return fail(nullptr, MTG_E_INVALID, "replica " + std::to_string(r) + ": replicas must share one force field");
        if(temperatures && !(temperatures[r] > 0.0)) return fail(nullptr, MTG_E_INVALID, "temperatures must be positive");
        if(cutoffs && !(cutoffs[r] > 0.0 && cutoffs[r] <= cfg->cutoff_radius))
            return fail(nullptr, MTG_E_INVALID, "replica cutoffs must be positive and at most cutoff_radius");
        N += s->n_atoms;
    }
    if(N > (long long)kIdxMask) return fail(nullptr, MTG_E_INVALID, "too many atoms in the batch");
    // merged system: atoms concatenated, molecule indices made distinct, topology offset
    BatchSpec bs;
    bs.nrep = nrep;
    std::vector<double> r3, p3, m, q;
    std::vector<int32_t> type, mol, bonds, angles, dihs;
    std::vector<uint8_t> mobile;
    double big[3] = {0.0, 0.0, 0.0};
    int off = 0, molbase = 0;
    for(int rr = 0; rr < nrep; rr++) {
        const mtg_system_desc* s = systems[rr];
        const int n = s->n_atoms;
        bs.off.push_back(off);
        bs.n.push_back(n);
        for(int a = 0; a < 3; a++) {
            bs.box.push_back(s->box[a]);
            big[a] = std::max(big[a], s->box[a]);
        }
        bs.temperature.push_back(temperatures ? temperatures[rr] : cfg->temperature);
        if(cutoffs) bs.cutoff.push_back(cutoffs[rr]);
        r3.insert(r3.end(), s->r, s->r + 3 * n);
        if(s->p) p3.insert(p3.end(), s->p, s->p + 3 * n);
        else p3.insert(p3.end(), (size_t)3 * n, 0.0);
        m.insert(m.end(), s->mass, s->mass + n);
        q.insert(q.end(), s->charge, s->charge + n);
        type.insert(type.end(), s->type, s->type + n);
        int mmax = -1;
        for(int i = 0; i < n; i++) {
            const int mi = s->mol ? s->mol[i] : -1;
            mol.push_back(mi >= 0 ? mi + molbase : -1);
            mmax = std::max(mmax, mi);
            mobile.push_back(s->mobile ? s->mobile[i] : 1);
        }
        molbase += mmax + 1;
        // a topology index must name an atom of its own replica: offset into the merged system,
        // an index in [n, N) would silently join atoms of different replicas
        auto add_topo = [&](std::vector<int32_t>& dst, int cnt, const int32_t* src, int w) -> bool {
            for(int j = 0; j < cnt; j++)
                for(int k = 0; k < w; k++) {
                    const int32_t v = src[w * j + k];
                    if(k < w - 1 && (v < 0 || v >= n)) return false;
                    dst.push_back(k < w - 1 ? v + off : v);
                }
            return true;
        };
        if((s->n_bonds > 0 && s->bonds && !add_topo(bonds, s->n_bonds, s->bonds, 3)) ||
           (s->n_angles > 0 && s->angles && !add_topo(angles, s->n_angles, s->angles, 4)) ||
           (s->n_dihedrals > 0 && s->dihedrals && !add_topo(dihs, s->n_dihedrals, s->dihedrals, 5))) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "replica %d: a bond, angle or dihedral index lies outside its %d atoms", rr, n);
            return fail(nullptr, MTG_E_INVALID, msg);
        }
        off += n;
    }
    bs.off.push_back(off);
    mtg_system_desc md = *s0;
    md.n_atoms = off;
    md.r = r3.data();
    md.p = p3.data();
    md.mass = m.data();
    md.charge = q.data();
    md.type = type.data();
    md.mol = mol.data();
    md.mobile = mobile.data();
    for(int a = 0; a < 3; a++) md.box[a] = big[a];
    md.n_bonds = (int32_t)(bonds.size() / 3);
    md.bonds = bonds.empty() ? nullptr : bonds.data();
    md.n_angles = (int32_t)(angles.size() / 4);
    md.angles = angles.empty() ? nullptr : angles.data();
    md.n_dihedrals = (int32_t)(dihs.size() / 5);
    md.dihedrals = dihs.empty() ? nullptr : dihs.data();
    return create_impl(&md, cfg, &bs, out);
}

int mtg_batch_info(mtg_ctx* c, int32_t* nrep, int32_t* offsets) {
    if(!c) return MTG_E_INVALID;
    if(nrep) *nrep = c->P.nrep;
    if(offsets)
        for(size_t r = 0; r < c->rep_off.size(); r++) offsets[r] = c->rep_off[r];
    return MTG_OK;
}

int mtg_batch_get_records(mtg_ctx* c, double* rec) {
    if(!c || !rec) return MTG_E_INVALID;
    if(!c->P.nrep) return fail(c, MTG_E_INVALID, "not a batch");
    if(c->h_rrec.size() != (size_t)8 * c->P.nrep) return fail(c, MTG_E_INVALID, "no output step yet");
    for(int r = 0; r < c->P.nrep; r++) {
        const double* x = &c->h_rrec[(size_t)8 * r];
        double* o = rec + 6 * r;
        o[0] = x[2];   // T
        o[1] = x[3];   // P
        o[2] = x[4];   // V
        o[3] = x[0];   // U
        o[4] = x[1];   // K
        o[5] = x[0] + x[1];
    }
    return MTG_OK;
}

int mtg_batch_set_thermo(mtg_ctx* c, int32_t rep, const mtg_thermo_state* th) {
    if(!c || !th) return MTG_E_INVALID;
    if(rep < 0 || rep >= c->P.nrep) return fail(c, MTG_E_INVALID, "replica index out of range");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    ThermoDev t{};
    CUDA_TRY(c, copy_now(c, &t, c->d.ths + rep, sizeof(t), cudaMemcpyDeviceToHost));
    const int M = std::min<int>(th->M, kMaxChain);
    for(int j = 0; j < M; j++) {
        t.eta[j] = th->eta[j];
        t.peta[j] = th->p_eta[j];
    }
    CUDA_TRY(c, copy_now(c, c->d.ths + rep, &t, sizeof(t), cudaMemcpyHostToDevice));
    CUDA_TRY(c, copy_now(c, c->d.ths_saved + rep, &t, sizeof(t), cudaMemcpyHostToDevice));
    return MTG_OK;
}

int mtg_batch_get_thermo(mtg_ctx* c, int32_t rep, mtg_thermo_state* th) {
    if(!c || !th) return MTG_E_INVALID;
    if(rep < 0 || rep >= c->P.nrep) return fail(c, MTG_E_INVALID, "replica index out of range");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    ThermoDev t{};
    CUDA_TRY(c, copy_now(c, &t, c->d.ths + rep, sizeof(t), cudaMemcpyDeviceToHost));
    std::memset(th, 0, sizeof(*th));
    th->M = c->P.M;
    for(int j = 0; j < c->P.M; j++) {
        th->eta[j] = t.eta[j];
        th->p_eta[j] = t.peta[j];
    }
    if(c->h_rep_box.size() == (size_t)3 * c->P.nrep)
        for(int a = 0; a < 3; a++) th->box[a] = c->h_rep_box[(size_t)3 * rep + a];
    return MTG_OK;
}

// ---------------------------------------------------------------------------------------------
// Force-field parameters and gradients
// ---------------------------------------------------------------------------------------------
}  // extern "C"

namespace {

// Device buffer freed with the scope.
struct DBuf {
    void* p = nullptr;
    ~DBuf() { if(p) cudaFree(p); }
    template<class T> T* as() { return static_cast<T*>(p); }
};
int dbuf(mtg_ctx* c, DBuf& b, size_t bytes) {
    if(cudaMalloc(&b.p, std::max<size_t>(bytes, 8)) != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(c, MTG_E_NOMEM, "gradient work buffer allocation failed");
    }
    cudaMemsetAsync(b.p, 0, std::max<size_t>(bytes, 8), c->stream);
    return MTG_OK;
}

// LJ term (first 12-6 / 12-8 entry) of type pair q, or -1.
int lj_slot(const mtg_ctx* c, int q) {
    for(int ff = 0; ff < c->h_nb_count[q]; ff++) {
        const int k = c->h_nb_terms[q * kMaxFF + ff].kind;
        if(k == MTG_NB_LJ || k == MTG_NB_LJ1208) return q * kMaxFF + ff;
    }
    return -1;
}

int check_param(mtg_ctx* c, const mtg_param& p) {
    const int T = c->P.T;
    switch(p.kind) {
    case MTG_P_LJ_EPS:
    case MTG_P_LJ_SIGMA:
        if(p.index < 0 || p.index >= T * T || lj_slot(c, p.index) < 0) return fail(c, MTG_E_INVALID, "no LJ term on that type pair");
        return MTG_OK;
    case MTG_P_CHARGE:
        if(!p.dq) return fail(c, MTG_E_INVALID, "charge parameter needs its dq direction");
        for(int i = 0; i < c->P.n; i++)
            if(p.dq[i] != 0.0) return MTG_OK;
        return fail(c, MTG_E_INVALID, "charge direction dq is zero");
    case MTG_P_BOND_K:
    case MTG_P_BOND_R0:
        if(p.index < 0 || p.index >= (int)c->h_bond_kind.size() || c->h_bond_kind[p.index] != MTG_BOND_HARM)
            return fail(c, MTG_E_INVALID, "bond parameters need a harmonic bond type");
        return MTG_OK;
    case MTG_P_ANGLE_K:
    case MTG_P_ANGLE_THETA0:
        if(p.index < 0 || p.index >= (int)c->h_angle_kind.size() || c->h_angle_kind[p.index] != MTG_ANGLE_HARM)
            return fail(c, MTG_E_INVALID, "angle parameters need a harmonic angle type");
        return MTG_OK;
    default:
        return fail(c, MTG_E_INVALID, "unknown parameter kind");
    }
}

// Device coefficients of an LJ term from (eps, sigma, alpha, rc) (as mtg_create packs them).
void lj_coef(const mtg_ctx* c, const mtg_term& t, double* co, double* fs) {
    const double s2 = t.p[1] * t.p[1], s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s12 = s6 * s6;
    co[0] = 4.0 * t.p[0] * s12;
    co[1] = 4.0 * t.p[0] * t.p[2] * (t.kind == MTG_NB_LJ ? s6 : s8);
    lj_shift_terms(t, co, c->cfg.cutoff_radius, c->cfg.lj_shift, &co[3], fs);
}

double get_param(const mtg_ctx* c, const mtg_param& p) {
    switch(p.kind) {
    case MTG_P_LJ_EPS: return c->h_nb_terms[lj_slot(c, p.index)].p[0];
    case MTG_P_LJ_SIGMA: return c->h_nb_terms[lj_slot(c, p.index)].p[1];
    case MTG_P_CHARGE:
        for(int i = 0; i < c->P.n; i++)
            if(p.dq[i] != 0.0) return c->h_charge[i] / p.dq[i];
        return 0.0;
    case MTG_P_BOND_K: return c->h_bond_par[4 * p.index];
    case MTG_P_BOND_R0: return c->h_bond_par[4 * p.index + 1];
    case MTG_P_ANGLE_K: return c->h_angle_par[4 * p.index];
    case MTG_P_ANGLE_THETA0: return c->h_angle_par[4 * p.index + 1] / c->h_angle_par[4 * p.index + 2];
    }
    return 0.0;
}

// Host-side parameter change; device arrays are refreshed by push_params.
void put_param(mtg_ctx* c, const mtg_param& p, double v) {
    const int T = c->P.T;
    switch(p.kind) {
    case MTG_P_LJ_EPS:
    case MTG_P_LJ_SIGMA: {
        const int r = p.index / T, col = p.index % T;
        for(int q : {r * T + col, col * T + r}) {
            const int slot = lj_slot(c, q);
            if(slot < 0) continue;
            c->h_nb_terms[slot].p[p.kind == MTG_P_LJ_EPS ? 0 : 1] = v;
            lj_coef(c, c->h_nb_terms[slot], &c->h_nb_coef[4 * slot], &c->h_nb_fs[slot]);
        }
        break;
    }
    case MTG_P_CHARGE:
        for(int i = 0; i < c->P.n; i++)
            if(p.dq[i] != 0.0) c->h_charge[i] = v * p.dq[i];
        break;
    case MTG_P_BOND_K: c->h_bond_par[4 * p.index] = v; break;
    case MTG_P_BOND_R0: c->h_bond_par[4 * p.index + 1] = v; break;
    case MTG_P_ANGLE_K: c->h_angle_par[4 * p.index] = v; break;
    case MTG_P_ANGLE_THETA0: c->h_angle_par[4 * p.index + 1] = v * c->h_angle_par[4 * p.index + 2]; break;
    }
}

int push_params(mtg_ctx* c) {
    DevSys& d = c->d;
    const int n = c->P.n;
    std::vector<float> f(c->h_nb_coef.begin(), c->h_nb_coef.end());
    CUDA_TRY(c, copy_now(c, (void*)d.nb_par, c->h_nb_coef.data(), c->h_nb_coef.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, copy_now(c, (void*)d.nb_parf, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    std::vector<float> fsf(c->h_nb_fs.begin(), c->h_nb_fs.end());
    CUDA_TRY(c, copy_now(c, (void*)d.nb_fs, c->h_nb_fs.data(), c->h_nb_fs.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(c, copy_now(c, (void*)d.nb_fsf, fsf.data(), fsf.size() * sizeof(float), cudaMemcpyHostToDevice));
    auto push = [&](const std::vector<double>& h, const double* dd, const float* df) -> int {
        std::vector<float> hf(h.begin(), h.end());
        CUDA_TRY(c, copy_now(c, (void*)dd, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
        CUDA_TRY(c, copy_now(c, (void*)df, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice));
        return MTG_OK;
    };
    int rc = push(c->h_bond_par, d.bond_par, d.bond_parf);
    rc = rc ? rc : push(c->h_angle_par, d.angle_par, d.angle_parf);
    if(rc) return rc;
    std::vector<float> qf(n);
    for(int i = 0; i < n; i++) qf[i] = (float)c->h_charge[i];
    CUDA_TRY(c, copy_now(c, d.qd, c->h_charge.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    CUDA_TRY(c, copy_now(c, d.qf, qf.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    // per-type charge table (and whether it describes every atom)
    const int T = c->P.T;
    std::vector<float> qt(std::max(T, 1), 0.0f);
    std::vector<int> seen(std::max(T, 1), 0);
    bool uniform = T <= 8;
    for(int i = 0; i < n && uniform; i++) {
        const int t = c->h_type[i];
        if(!seen[t]) { seen[t] = 1; qt[t] = qf[i]; }
        else if(qt[t] != qf[i]) uniform = false;
    }
    CUDA_TRY(c, copy_now(c, (void*)d.qtype, qt.data(), sizeof(float) * qt.size(), cudaMemcpyHostToDevice));
    if((uniform ? 1 : 0) != c->P.qtype) {
        c->P.qtype = uniform ? 1 : 0;
        c->generation++;   // captured graphs hold the old flag
    }
    const int qany = any_charge(c);
    if(qany != c->P.qany) {
        c->P.qany = qany;
        c->generation++;
    }
    const int qon = charges_on(c);
    if(qon != c->P.qon) {
        c->P.qon = qon;
        c->generation++;
        // charges switched on: the list must reach rcoul for every pair
        if(!is_reference(c)) cudaMemsetAsync(&c->d.sc->rebuild, 0xff, sizeof(int32_t), c->stream);
    }
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncFromMaster, c->stream);   // charges also live in hi.w
    return MTG_OK;
}

// Tangent tables of parameter p (host vectors sized like the device ones), uploaded to buf.
struct TangentSet {
    DBuf nb, fs, q, bond, angle;
    AdjTangents t{};
};
int make_tangents(mtg_ctx* c, const mtg_param& p, TangentSet& ts) {
    const int T = c->P.T, n = c->P.n;
    ts.t = AdjTangents{};
    switch(p.kind) {
    case MTG_P_LJ_EPS:
    case MTG_P_LJ_SIGMA: {
        // a = 4 eps sigma^12, b = 4 eps alpha sigma^n are linear in eps and powers of sigma; the
        // cutoff constants (energy shift, force at the cutoff) are linear in (a, b)
        std::vector<double> nt(c->h_nb_coef.size(), 0.0), ft(c->h_nb_fs.size(), 0.0);
        const int r = p.index / T, col = p.index % T;
        for(int q : {r * T + col, col * T + r}) {
            const int slot = lj_slot(c, q);
            if(slot < 0) continue;
            const mtg_term& tm = c->h_nb_terms[slot];
            const double e = tm.p[0], sg = tm.p[1], al = tm.p[2];
            const double nn = tm.kind == MTG_NB_LJ ? 6.0 : 8.0;
            double co_t[4] = {0.0, 0.0, 0.0, 0.0};
            if(p.kind == MTG_P_LJ_EPS) {
                co_t[0] = 4.0 * std::pow(sg, 12.0);
                co_t[1] = 4.0 * al * std::pow(sg, nn);
            } else {
                co_t[0] = 48.0 * e * std::pow(sg, 11.0);
                co_t[1] = 4.0 * e * al * nn * std::pow(sg, nn - 1.0);
            }
            double us_t, fs_t;
            lj_shift_terms(tm, co_t, c->cfg.cutoff_radius, c->cfg.lj_shift, &us_t, &fs_t);
            nt[4 * slot] = co_t[0];
            nt[4 * slot + 1] = co_t[1];
            nt[4 * slot + 3] = us_t;
            ft[slot] = fs_t;
        }
        int rc = dbuf(c, ts.nb, nt.size() * sizeof(double));
        if(!rc) rc = dbuf(c, ts.fs, ft.size() * sizeof(double));
        if(rc) return rc;
        CUDA_TRY(c, copy_now(c, ts.nb.p, nt.data(), nt.size() * sizeof(double), cudaMemcpyHostToDevice));
        CUDA_TRY(c, copy_now(c, ts.fs.p, ft.data(), ft.size() * sizeof(double), cudaMemcpyHostToDevice));
        ts.t.nb_par_t = ts.nb.as<double>();
        ts.t.nb_fs_t = ts.fs.as<double>();
        return MTG_OK;
    }
    case MTG_P_CHARGE: {
        int rc = dbuf(c, ts.q, sizeof(double) * n);
        if(rc) return rc;
        CUDA_TRY(c, copy_now(c, ts.q.p, p.dq, sizeof(double) * n, cudaMemcpyHostToDevice));
        ts.t.q_t = ts.q.as<double>();
        return MTG_OK;
    }
    case MTG_P_BOND_K:
    case MTG_P_BOND_R0: {
        std::vector<double> bt(c->h_bond_par.size(), 0.0);
        bt[4 * p.index + (p.kind == MTG_P_BOND_K ? 0 : 1)] = 1.0;
        int rc = dbuf(c, ts.bond, bt.size() * sizeof(double));
        if(rc) return rc;
        CUDA_TRY(c, copy_now(c, ts.bond.p, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice));
        ts.t.bond_par_t = ts.bond.as<double>();
        return MTG_OK;
    }
    case MTG_P_ANGLE_K:
    case MTG_P_ANGLE_THETA0: {
        std::vector<double> at(c->h_angle_par.size(), 0.0);
        if(p.kind == MTG_P_ANGLE_K) at[4 * p.index] = 1.0;
        else at[4 * p.index + 1] = c->h_angle_par[4 * p.index + 2];   // d(theta0 rad)/d(theta0 deg)
        int rc = dbuf(c, ts.angle, at.size() * sizeof(double));
        if(rc) return rc;
        CUDA_TRY(c, copy_now(c, ts.angle.p, at.data(), at.size() * sizeof(double), cudaMemcpyHostToDevice));
        ts.t.angle_par_t = ts.angle.as<double>();
        return MTG_OK;
    }
    }
    return MTG_E_INVALID;
}

// FP64 positions of the current state in d.r (mixed: assembled from hi + lo).
void positions_to_r(mtg_ctx* c) {
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncToMaster, c->stream);
}

// Places FP64 positions `pos` as the current positions and rebuilds the Verlet list there.
void place_positions(mtg_ctx* c, const double* pos) {
    if(pos != c->d.r)
        cudaMemcpyAsync(c->d.r, pos, sizeof(double) * 3 * c->P.n, cudaMemcpyDeviceToDevice, c->stream);
    if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncPositionsFromMaster, c->stream);
    launch_prod_build(c->d, c->P, true, c->stream);
}

// Ordered sum of x.y over n entries (device partials, host total).
int dot(mtg_ctx* c, int n, const double* x, const double* y, DBuf& part, double* out) {
    const int nb = dot_blocks(n);
    launch_dot_blocks(n, x, y, part.as<double>(), c->stream);
    std::vector<double> h(nb);
    CUDA_TRY(c, cudaMemcpyAsync(h.data(), part.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    double s = 0.0;
    for(double v : h) s += v;
    *out = s;
    return MTG_OK;
}

int grad_preflight(mtg_ctx* c, int32_t np, const mtg_param* params, bool batch = false) {
    if(is_reference(c)) return fail(c, MTG_E_UNSUPPORTED, "gradients use the analytic terms of the fp64 / mixed modes");
    if(c->P.nrep && !batch) return fail(c, MTG_E_UNSUPPORTED, "a batch takes its gradients per replica (mtg_batch_energy_grad)");
    if(c->P.ensemble == MTG_NPT) return fail(c, MTG_E_UNSUPPORTED, "gradients are taken at a fixed box (NVT or NVE)");
    if(!c->P.nrep && batch) return fail(c, MTG_E_INVALID, "not a batch");
    if(c->has_tables) return fail(c, MTG_E_UNSUPPORTED, "tabulated terms have no derivative");
    if(np < 0 || (np > 0 && !params)) return MTG_E_INVALID;
    for(int k = 0; k < np; k++) {
        int rc = check_param(c, params[k]);
        if(rc) return rc;
    }
    return MTG_OK;
}

}  // namespace

extern "C" {

int mtg_get_params(mtg_ctx* c, int32_t np, const mtg_param* params, double* values) {
    if(!c || !values) return MTG_E_INVALID;
    for(int k = 0; k < np; k++) {
        int rc = check_param(c, params[k]);
        if(rc) return rc;
        values[k] = get_param(c, params[k]);
    }
    return MTG_OK;
}

int mtg_set_params(mtg_ctx* c, int32_t np, const mtg_param* params, const double* values) {
    if(!c || !values) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    if(is_reference(c)) return fail(c, MTG_E_UNSUPPORTED, "the reference mode keeps its tables; set parameters in fp64 / mixed");
    int rc = settle_state(c);
    if(rc) return rc;
    for(int k = 0; k < np; k++) {
        rc = check_param(c, params[k]);
        if(rc) return rc;
        if(!std::isfinite(values[k])) return fail(c, MTG_E_NONFINITE, "non-finite parameter value");
    }
    for(int k = 0; k < np; k++) put_param(c, params[k], values[k]);
    rc = push_params(c);
    if(rc) return rc;
    return compute_forces_now(c, true);
}

int mtg_energy_grad(mtg_ctx* c, int32_t np, const mtg_param* params, double* U, double* grad) {
    if(!c) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = grad_preflight(c, np, params);
    if(rc) return rc;
    rc = settle_state(c);
    if(rc) return rc;
    const int n = c->P.n;
    positions_to_r(c);
    place_positions(c, c->d.r);
    launch_prod_force(c->d, c->P, true, c->stream);
    if(is_mixed(c)) launch_prod_forces_to_double(c->d, c->P, c->stream);
    DBuf Ft, Ut, part;
    if((rc = dbuf(c, Ft, sizeof(double) * 3 * n)) || (rc = dbuf(c, Ut, sizeof(double) * n)) ||
       (rc = dbuf(c, part, sizeof(double) * dot_blocks(3 * n))))
        return rc;
    if(U) {
        rc = dot(c, n, c->d.U, nullptr, part, U);
        if(rc) return rc;
    }
    for(int k = 0; k < np; k++) {
        TangentSet ts;
        rc = make_tangents(c, params[k], ts);
        if(rc) return rc;
        launch_force_tangent(c->d, c->P, c->d.r, ts.t, Ft.as<double>(), Ut.as<double>(), c->stream);
        CUDA_TRY(c, cudaGetLastError());
        rc = dot(c, n, Ut.as<double>(), nullptr, part, &grad[k]);
        if(rc) return rc;
    }
    return MTG_OK;
}

int mtg_batch_energy_grad(mtg_ctx* c, int32_t np, const mtg_param* params, double* U, double* grad) {
    if(!c || (np > 0 && !grad)) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = grad_preflight(c, np, params, true);
    if(rc) return rc;
    rc = settle_state(c);
    if(rc) return rc;
    const int n = c->P.n, nr = c->P.nrep;
    positions_to_r(c);
    place_positions(c, c->d.r);
    launch_prod_force(c->d, c->P, true, c->stream);
    if(is_mixed(c)) launch_prod_forces_to_double(c->d, c->P, c->stream);
    DBuf Ft, Ut, off, sums;
    if((rc = dbuf(c, Ft, sizeof(double) * 3 * n)) || (rc = dbuf(c, Ut, sizeof(double) * n)) ||
       (rc = dbuf(c, off, sizeof(int) * (nr + 1))) || (rc = dbuf(c, sums, sizeof(double) * nr * (np + 1))))
        return rc;
    CUDA_TRY(c, cudaMemcpyAsync(off.p, c->rep_off.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice, c->stream));
    double* sm = sums.as<double>();
    launch_segment_sums(c->d.U, off.as<int>(), nr, sm, c->stream);
    for(int k = 0; k < np; k++) {
        TangentSet ts;
        rc = make_tangents(c, params[k], ts);
        if(rc) return rc;
        launch_force_tangent(c->d, c->P, c->d.r, ts.t, Ft.as<double>(), Ut.as<double>(), c->stream);
        launch_segment_sums(Ut.as<double>(), off.as<int>(), nr, sm + (size_t)nr * (k + 1), c->stream);
        CUDA_TRY(c, cudaGetLastError());
    }
    std::vector<double> h((size_t)nr * (np + 1));
    CUDA_TRY(c, cudaMemcpyAsync(h.data(), sm, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for(int r = 0; r < nr; r++) {
        if(U) U[r] = h[r];
        for(int k = 0; k < np; k++) grad[(size_t)r * np + k] = h[(size_t)nr * (k + 1) + r];
    }
    return MTG_OK;
}

int mtg_loss_grad(mtg_ctx* c, const mtg_loss_desc* L, int32_t np, const mtg_param* params, double* loss, double* grad,
                  double* rdf) {
    if(!c || !L || !L->target) return MTG_E_INVALID;
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = grad_preflight(c, np, params);
    if(rc) return rc;
    const int T = c->P.T, n = c->P.n, n3 = 3 * n;
    const int S = L->nsteps, K = L->checkpoint_every > 0 ? L->checkpoint_every : L->nsteps;
    if(S < 1 || L->nbins < 1 || !(L->rmax > 0.0) || !(L->width > 0.0) || L->type_a < 0 || L->type_a >= T ||
       L->type_b < 0 || L->type_b >= T)
        return fail(c, MTG_E_INVALID, "bad loss description");
    const double rlist = std::max((double)c->P.rc, (double)c->P.rcoul) + c->P.skin;
    if(L->rmax + 8.0 * L->width > rlist) return fail(c, MTG_E_INVALID, "rmax + 8 width must lie inside the Verlet-list radius");
    rc = settle_state(c);
    if(rc) return rc;
    // the differentiated trajectory is plain velocity Verlet (NVE, no force clipping)
    const Params saved = c->P;
    struct Restore {
        mtg_ctx* c;
        Params P;
        ~Restore() {
            if(c->P.ensemble != P.ensemble || c->P.M != P.M || c->P.clip != P.clip) c->generation++;
            c->P = P;
            // per-pair list radii again (the current list keeps the loss pair's extra partners,
            // which the force kernels skip by their cutoffs, until the next rebuild)
            (void)upload_pair_cuts(c, -1, -1);
        }
    } restore{c, saved};
    // the loss pair's partners out to the full list radius (the rebuild below places them)
    rc = upload_pair_cuts(c, L->type_a, L->type_b);
    if(rc) return rc;
    c->P.ensemble = MTG_NVE;
    c->P.M = 0;
    c->P.clip = 0;
    const int nck = (S + K - 1) / K + 1;
    DBuf ck_r, ck_p, seg, rows, hist, lam_r, lam_v, Ft, part, invm, cb, r0, p0;
    if((rc = dbuf(c, ck_r, sizeof(double) * n3 * nck)) || (rc = dbuf(c, ck_p, sizeof(double) * n3 * nck)) ||
       (rc = dbuf(c, seg, sizeof(double) * n3 * (K + 1))) || (rc = dbuf(c, rows, sizeof(double) * n * L->nbins)) ||
       (rc = dbuf(c, hist, sizeof(double) * L->nbins)) || (rc = dbuf(c, lam_r, sizeof(double) * n3)) ||
       (rc = dbuf(c, lam_v, sizeof(double) * n3)) || (rc = dbuf(c, Ft, sizeof(double) * n3)) ||
       (rc = dbuf(c, part, sizeof(double) * dot_blocks(n3))) || (rc = dbuf(c, invm, sizeof(double) * n)) ||
       (rc = dbuf(c, cb, sizeof(double) * L->nbins)) || (rc = dbuf(c, r0, sizeof(double) * n3)) ||
       (rc = dbuf(c, p0, sizeof(double) * n3)))
        return rc;
    {
        // 1/m for mobile atoms, 0 for immobile ones (their positions never change)
        std::vector<double> im(n);
        std::vector<int> mob(n);
        CUDA_TRY(c, copy_now(c, mob.data(), c->d.mobile, sizeof(int) * n, cudaMemcpyDeviceToHost));
        for(int i = 0; i < n; i++) im[i] = mob[i] ? 1.0 / c->h_mass[i] : 0.0;
        CUDA_TRY(c, copy_now(c, invm.p, im.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    }
    AdjRdf rs{L->type_a, L->type_b, L->nbins, L->rmax, L->width};
    const double dt = c->P.dt;
    double* R = c->d.r;
    // initial state
    positions_to_r(c);
    CUDA_TRY(c, cudaMemcpyAsync(r0.p, R, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(p0.p, c->d.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
    auto restore_state = [&](const double* r, const double* p) -> int {
        CUDA_TRY(c, cudaMemcpyAsync(c->d.p, p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
        place_positions(c, r);
        if(is_mixed(c)) launch_prod_sync(c->d, c->P, kSyncFromMaster, c->stream);
        int rc2 = compute_forces_now(c, false);
        if(rc2) return rc2;
        launch_prologue(c->d, c->P, c->stream);   // pending scale S = 1 (NVE)
        return MTG_OK;
    };
    auto step = [&]() -> int {
        launch_prod_kick_drift(c->d, c->P, c->stream);
        launch_prod_build(c->d, c->P, false, c->stream);
        launch_prod_force(c->d, c->P, false, c->stream);
        launch_prod_kick2(c->d, c->P, false, c->stream);
        positions_to_r(c);
        CUDA_TRY(c, cudaGetLastError());
        return MTG_OK;
    };
    // ---- forward: checkpoints every K steps, pair correlation after every step ----
    for(int attempt = 0;; attempt++) {
        clear_overflow(c);
        rc = restore_state(r0.as<double>(), p0.as<double>());
        if(rc) return rc;
        CUDA_TRY(c, cudaMemsetAsync(hist.p, 0, sizeof(double) * L->nbins, c->stream));
        for(int t = 0; t < S; t++) {
            if(t % K == 0) {
                CUDA_TRY(c, cudaMemcpyAsync(ck_r.as<double>() + (size_t)(t / K) * n3, R, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
                CUDA_TRY(c, cudaMemcpyAsync(ck_p.as<double>() + (size_t)(t / K) * n3, c->d.p, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
            }
            rc = step();
            if(rc) return rc;
            launch_rdf_rows(c->d, c->P, R, rs, rows.as<double>(), c->stream);
            launch_rdf_reduce(rows.as<double>(), n, L->nbins, hist.as<double>(), c->stream);
        }
        StepScalars sc = read_scalars(c);
        if(!sc.overflow) break;
        if(attempt > 8) return fail(c, MTG_E_OVERFLOW, "neighbour list did not converge");
        rc = grow_vlist(c, sc.needed);
        if(rc) return rc;
    }
    // ---- loss ----
    std::vector<double> h(L->nbins), norm(L->nbins), gbar(L->nbins), w(L->nbins);
    CUDA_TRY(c, copy_now(c, h.data(), hist.p, sizeof(double) * L->nbins, cudaMemcpyDeviceToHost));
    long long na = 0, nb = 0;
    for(int i = 0; i < n; i++) {
        na += (c->h_type[i] == L->type_a);
        nb += (c->h_type[i] == L->type_b);
    }
    const double npairs = (L->type_a == L->type_b) ? 0.5 * double(na) * double(na - 1) : double(na) * double(nb);
    const double V = c->P.box[0] * c->P.box[1] * c->P.box[2];
    const double dr = L->rmax / L->nbins;
    double Lval = 0.0;
    for(int b = 0; b < L->nbins; b++) {
        const double x = (b + 0.5) * dr;
        norm[b] = (npairs > 0.0) ? V / (npairs * 4.0 * M_PI * x * x) : 0.0;
        gbar[b] = norm[b] * h[b] / S;
        const double dev = gbar[b] - L->target[b];
        Lval += dev * dev;
        w[b] = 2.0 * dev / S * norm[b];   // dL/d(sum_pairs K(r - x_b)) at each frame
    }
    if(loss) *loss = Lval;
    if(rdf) std::memcpy(rdf, gbar.data(), sizeof(double) * L->nbins);
    CUDA_TRY(c, copy_now(c, cb.p, w.data(), sizeof(double) * L->nbins, cudaMemcpyHostToDevice));
    if(np == 0 || !grad) {
        rc = restore_state(r0.as<double>(), p0.as<double>());
        if(rc) return rc;
        return compute_forces_now(c, true);
    }
    // ---- backward: leapfrog adjoint, segment by segment from the last checkpoint ----
    std::vector<TangentSet> ts(np);
    for(int k = 0; k < np; k++) {
        rc = make_tangents(c, params[k], ts[k]);
        if(rc) return rc;
    }
    DBuf gdev;   // gradient accumulated on the device, read once at the end
    if((rc = dbuf(c, gdev, sizeof(double) * np))) return rc;
    double* lr = lam_r.as<double>();
    double* lv = lam_v.as<double>();
    AdjTangents hv{};
    hv.vpos = lv;
    bool first = true;
    for(int s0 = ((S - 1) / K) * K; s0 >= 0; s0 -= K) {
        const int s1 = std::min(s0 + K, S);
        rc = restore_state(ck_r.as<double>() + (size_t)(s0 / K) * n3, ck_p.as<double>() + (size_t)(s0 / K) * n3);
        if(rc) return rc;
        double* sg = seg.as<double>();
        CUDA_TRY(c, cudaMemcpyAsync(sg, R, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
        for(int t = s0 + 1; t <= s1; t++) {
            rc = step();
            if(rc) return rc;
            CUDA_TRY(c, cudaMemcpyAsync(sg + (size_t)(t - s0) * n3, R, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
        }
        for(int t = s1; t > s0; t--) {
            const double* pt = sg + (size_t)(t - s0) * n3;
            const double* pm = sg + (size_t)(t - 1 - s0) * n3;
            if(first) {
                // lambda_r = dL/dr_S
                place_positions(c, pt);
                launch_rdf_adjoint(c->d, c->P, R, rs, cb.as<double>(), lr, c->stream);
                first = false;
            }
            launch_axpy(n3, dt, lr, invm.as<double>(), lv, c->stream);          // lambda_v += dt lambda_r / m
            place_positions(c, pm);
            const double wk = (t - 1 >= 1) ? dt : 0.5 * dt;
            launch_force_tangent(c->d, c->P, R, hv, Ft.as<double>(), nullptr, c->stream);
            launch_axpy(n3, wk, Ft.as<double>(), nullptr, lr, c->stream);       // lambda_r += w J lambda_v
            for(int k = 0; k < np; k++) {
                launch_force_tangent(c->d, c->P, R, ts[k].t, Ft.as<double>(), nullptr, c->stream);
                launch_dot_accum(n3, lv, Ft.as<double>(), wk, part.as<double>(), gdev.as<double>() + k, c->stream);
            }
            if(t - 1 >= 1) launch_rdf_adjoint(c->d, c->P, R, rs, cb.as<double>(), lr, c->stream);
            CUDA_TRY(c, cudaGetLastError());
        }
    }
    CUDA_TRY(c, cudaMemcpyAsync(grad, gdev.p, sizeof(double) * np, cudaMemcpyDeviceToHost, c->stream));
    // back to the initial state
    rc = restore_state(r0.as<double>(), p0.as<double>());
    if(rc) return rc;
    rc = compute_forces_now(c, true);
    if(rc) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MTG_OK;
}

int mtg_pair_histogram(mtg_ctx* c, int32_t type_a, int32_t type_b, int32_t nbins, double rmin, double rmax,
                       double ignore_below, int64_t* profile) {
    if(!c || !profile || nbins < 1 || nbins > 8192 || !(rmax != rmin)) return MTG_E_INVALID;
    if(c->P.nrep) return fail(c, MTG_E_UNSUPPORTED, "pair histograms are taken per system");
    if(type_a < 0 || type_a >= c->P.T || type_b < 0 || type_b >= c->P.T) return fail(c, MTG_E_INVALID, "type out of range");
    CUDA_TRY(c, cudaSetDevice(c->device));
    int rc = settle_state(c);
    if(rc) return rc;
    std::vector<int> ia, ib;
    for(int i = 0; i < c->P.n; i++) {
        if(c->h_type[i] == type_a) ia.push_back(i);
        if(c->h_type[i] == type_b) ib.push_back(i);
    }
    if(ia.empty() || ib.empty()) return MTG_OK;
    DBuf dia, dib, prof;
    if((rc = dbuf(c, dia, sizeof(int) * ia.size())) || (rc = dbuf(c, dib, sizeof(int) * ib.size())) ||
       (rc = dbuf(c, prof, sizeof(unsigned long long) * nbins)))
        return rc;
    CUDA_TRY(c, cudaMemcpyAsync(dia.p, ia.data(), sizeof(int) * ia.size(), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(dib.p, ib.data(), sizeof(int) * ib.size(), cudaMemcpyHostToDevice, c->stream));
    positions_to_r(c);
    double box[3] = {c->P.box[0], c->P.box[1], c->P.box[2]};
    if(c->P.ensemble == MTG_NPT) {
        BaroDev b{};
        CUDA_TRY(c, copy_now(c, &b, c->d.baro, sizeof(b), cudaMemcpyDeviceToHost));
        for(int a = 0; a < 3; a++) box[a] = b.L[a];
    }
    launch_pair_hist(c->d.r, dia.as<int>(), (int)ia.size(), dib.as<int>(), (int)ib.size(), box, rmin, rmax, nbins, ignore_below,
                     prof.as<unsigned long long>(), c->stream);
    CUDA_TRY(c, cudaGetLastError());
    std::vector<unsigned long long> h(nbins);
    CUDA_TRY(c, cudaMemcpyAsync(h.data(), prof.p, sizeof(unsigned long long) * nbins, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for(int b = 0; b < nbins; b++) profile[b] += (int64_t)h[b];
    return MTG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// No-allocation neighbour list: the reference-order cell list and neighbour list kernels run on
// caller-owned positions and outputs, with their working arrays carved out of one file-scope
// device array instead of cudaMalloc'ed buffers.
// ---------------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[MTG_NOALLOC_SCRATCH_BYTES];

namespace {

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// Address of g_noalloc_scratch in the current device's context, looked up on every call.  The
// lookup is a host-side table read once the module is loaded; caching it per device number would
// go stale when the caller resets the device or makes another context current.  The first call on
// a device also loads this library's module there.
cudaError_t noalloc_scratch(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if(e == cudaSuccess) *out = p;
    return e;
}

// True when p is device (or managed) memory usable by device `dev`.
bool on_device(const void* p, int dev) {
    cudaPointerAttributes a{};
    if(cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if(a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" int mtg_neighbors_noalloc(const double* d_r, int32_t n, const double box[3], double cutoff, double shell,
                                     int32_t max_neigh, int32_t* d_count, int32_t* d_list, int32_t* needed,
                                     void* stream) {
    g_create_error.clear();
    if(!d_r || !box || !d_count || n <= 0 || max_neigh < 0 || (max_neigh > 0 && !d_list))
        return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: null pointer or non-positive size");
    if(n > (int32_t)kIdxMask) return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: too many atoms");
    if(!(cutoff > 0.0) || !(shell >= 0.0) || !std::isfinite(cutoff) || !std::isfinite(shell))
        return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: cutoff must be positive and shell non-negative");
    int cells[3];
    long long ncell = 1;
    for(int a = 0; a < 3; a++) {
        if(!(box[a] > 0.0) || !std::isfinite(box[a])) return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: box edges must be positive");
        const double nc = std::floor(double((float)box[a] / ((float)cutoff + (float)shell)));
        if(nc < 1.0) return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: box narrower than cutoff + shell");
        if(nc > 1048576.0) return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: too many cells for the scratch array");
        cells[a] = (int)nc;
        ncell *= (long long)nc;
    }
    const size_t b_sc = round256(sizeof(StepScalars));
    const size_t b_atom_cell = round256(sizeof(int) * 3 * (size_t)n);
    const size_t b_cell = round256(sizeof(int) * (size_t)ncell);
    const size_t b_list = round256(sizeof(int) * (size_t)n);
    const size_t need_bytes = b_sc + b_atom_cell + 3 * b_cell + b_list;
    if(ncell > (1LL << 30) || need_bytes > (size_t)MTG_NOALLOC_SCRATCH_BYTES) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "mtg_neighbors_noalloc: %d atoms in %lld cells need %zu bytes of scratch, the array holds %u; "
                      "use mtg_create/mtg_get_neighbors for this system",
                      n, ncell, need_bytes, (unsigned)MTG_NOALLOC_SCRATCH_BYTES);
        return fail(nullptr, MTG_E_INVALID, msg);
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if(e != cudaSuccess || dev < 0) {
        (void)cudaGetLastError();
        return fail(nullptr, MTG_E_CUDA, "mtg_neighbors_noalloc: no current CUDA device");
    }
    if(!on_device(d_r, dev) || !on_device(d_count, dev) || (d_list && !on_device(d_list, dev)))
        return fail(nullptr, MTG_E_INVALID, "mtg_neighbors_noalloc: d_r, d_count and d_list must be device memory of the current device");
    void* base = nullptr;
    e = noalloc_scratch(&base);
    if(e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(nullptr, MTG_E_CUDA, std::string("mtg_neighbors_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    }
    unsigned char* p = static_cast<unsigned char*>(base);
    DevSys d{};
    d.n = n;
    d.r = const_cast<double*>(d_r);
    d.sc = reinterpret_cast<StepScalars*>(p);
    p += b_sc;
    d.atom_cell = reinterpret_cast<int*>(p);
    p += b_atom_cell;
    d.cell_first = reinterpret_cast<int*>(p);
    p += b_cell;
    d.cell_count = reinterpret_cast<int*>(p);
    p += b_cell;
    d.cell_cursor = reinterpret_cast<int*>(p);
    p += b_cell;
    d.cell_list = reinterpret_cast<int*>(p);
    d.nbr_count = d_count;     // also the cell scatter's temporary, rewritten by the list kernel
    d.nbr_list = d_list;
    d.nbr_max = max_neigh;
    Params P{};
    P.n = n;
    for(int a = 0; a < 3; a++) {
        P.box[a] = box[a];
        P.boxf[a] = (float)box[a];
    }
    P.nx = cells[0];
    P.ny = cells[1];
    P.nz = cells[2];
    P.rc = (float)cutoff;
    P.shell = (float)shell;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Only the list kernel's overflow flag and maximum start at zero; the cell counts are cleared
    // by the cell-list launch itself, every other array is written before it is read.
    e = cudaMemsetAsync(d.sc, 0, sizeof(StepScalars), s);
    if(e == cudaSuccess) {
        launch_ref_cells(d, P, s);
        launch_ref_neigh(d, P, s);
        e = cudaGetLastError();
    }
    if(e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(nullptr, MTG_E_CUDA, std::string("mtg_neighbors_noalloc: ") + cudaGetErrorString(e));
    }
    if(needed) {
        int32_t mx[2] = {0, 0};   // StepScalars::overflow, StepScalars::needed
        e = cudaMemcpyAsync(mx, &d.sc->overflow, sizeof mx, cudaMemcpyDeviceToHost, s);
        if(e == cudaSuccess) e = cudaStreamSynchronize(s);
        if(e != cudaSuccess) {
            (void)cudaGetLastError();
            return fail(nullptr, MTG_E_CUDA, std::string("mtg_neighbors_noalloc: ") + cudaGetErrorString(e));
        }
        *needed = mx[0] ? mx[1] : 0;
    }
    return MTG_OK;
}
