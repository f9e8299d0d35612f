/*
 * mtgpu.h -- C ABI of libmtgpu.so, the GB300-native (sm_103a) molecular-dynamics engine that
 * replaces the engine behind MolTwister's `moldyn run`.
 *
 * What it replaces.  In the reference, `CCmdRun::execute` (Cmd/MolTwisterCmdMolDyn/CmdRun.cpp:84-139)
 * hands the whole CMolTwisterState to `mtdev::CMDSimulator::run(SMolDynConfigStruct, FILE*,
 * CSerializer&)` (Simulator/MDSimulator.h:33-43, MDSimulator.cpp:28-47), which builds
 * CSimulationBox/CMDLoop and runs velocity-Verlet + Nose-Hoover with forces from
 * CMDFFMatrices + CFunctorCalcForce.  Here the caller describes the system once
 * (mtg_system_desc: atoms plus the MDFF term tables and parameters) and the run settings
 * (mtg_config_desc: the SMolDynConfigStruct fields the engine reads), then steps it on the GPU.
 *
 * Conventions.
 *   - Every function returns MTG_OK (0) or a negative MTG_E* code; mtg_last_error() gives a
 *     message.  No C++ exception crosses this boundary.
 *   - The caller owns every host array it passes; the library copies what it needs and owns all
 *     device memory of a context.
 *   - A context is not re-entrant: call it from one thread at a time.  Distinct contexts may be
 *     used from distinct threads.
 *   - Units are the reference's (Integrators/Constants.h:23-40): A, g/mol, kJ/mol, e; momenta
 *     p = m v with v in A per 100 fs; temperatures in K; times in fs.
 *   - The periodic box spans [-L/2, L/2) on each axis, as CCellList::updatePBC assumes
 *     (MDFFMatrices.cpp:67-76).
 *   - Any wait inside a device kernel is bounded and reports MTG_E_TIMEOUT.
 */
#ifndef MTGPU_H
#define MTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MTG_ABI_VERSION 1

/* Return codes */
#define MTG_OK 0
#define MTG_E_INVALID (-1)    /* bad argument or inconsistent descriptor */
#define MTG_E_CUDA (-2)       /* CUDA runtime error (message holds cudaGetErrorString) */
#define MTG_E_NOMEM (-3)      /* device or host allocation failed */
#define MTG_E_OVERFLOW (-4)   /* a list could not be grown to hold its entries */
#define MTG_E_TIMEOUT (-5)    /* a bounded device wait gave up */
#define MTG_E_UNSUPPORTED (-6)/* valid request this build does not implement */
#define MTG_E_NONFINITE (-7)  /* NaN/Inf in inputs or in the integrated state */

/* Points per tabulated 1D force/potential profile (MDFFMatrices.h:27) and non-bonded terms per
 * atom-type pair (MDFFMatrices.h:26). */
#define MTG_NPTS 1000
#define MTG_MAX_FF_PER_PAIR 5
#define MTG_MAX_NH_CHAIN 16

/* Term kinds.  Parameters follow the reference classes' parse order (see mtg_term). */
#define MTG_KIND_NONE 0
#define MTG_NB_LJ 1           /* p = {epsilon, sigma, alpha, rc}     MolTwisterMDFFNonBonded_LJ.cpp:131-162 */
#define MTG_NB_LJ1208 2       /* p = {epsilon, sigma, alpha, rc}     MolTwisterMDFFNonBonded_LJ1208.cpp:131-170 */
/* rc (new, production modes only): cutoff of this pair term, 0 = cutoff_radius.  The reference
 * has one global cutoff, so per-pair cutoffs (e.g. 2.5 sigma_ab of a binary mixture) are not
 * expressible there; reference mode ignores rc. */
#define MTG_NB_BUCK 3         /* p = {A, rho, C}                     MolTwisterMDFFNonBonded_Buck.cpp:116-143 */
#define MTG_NB_LJBUCK 4       /* table only                          MolTwisterMDFFNonBonded_LJBuck.cpp:181-251 */
#define MTG_BOND_HARM 11      /* p = {k, r0}, U = k (r - r0)^2       MolTwisterMDFFBond_Harm.cpp:90-110 */
#define MTG_BOND_MORSE 12     /* p = {D, alpha, r0}                  MolTwisterMDFFBond_Morse.cpp:95-117 */
#define MTG_BOND_LJC 13       /* table only (zero force)             MolTwisterMDFFBond_LJC.cpp */
#define MTG_ANGLE_HARM 21     /* p = {k, theta0 [deg], toRad}        MolTwisterMDFFAngle_Harm.cpp:94-130 */
#define MTG_ANGLE_CLASS2 22   /* table only                          MolTwisterMDFFAngle_Class2.cpp:145-296 */
#define MTG_DIH_HARM 31       /* p = {K, D, N}, U = K(1 + D cos N phi) MolTwisterMDFFDih_Harm.cpp:96-132 */
#define MTG_DIH_FOURIER4T 32  /* p = {V1, V2, V3, V4}                MolTwisterMDFFDih_Fourier4t.cpp:98-142 */

/* Precision modes (new key `precision`; the reference has only its own arithmetic). */
#define MTG_PREC_REFERENCE 0  /* reference semantics: 1000-point FP32 tables, FP64 accumulation,
                                 cell + neighbour lists rebuilt every step with the reference's
                                 order, all-pairs minimum-image Coulomb.  The parity mode. */
#define MTG_PREC_FP64 1       /* analytic terms in FP64, Verlet list with skin */
#define MTG_PREC_MIXED 2      /* analytic terms in FP32, forces summed as int64 fixed point
                                 (deterministic), positions, momenta and the thermostat chain as
                                 double-float (FP32 hi+lo) pairs, FP64 system sums */

/* Coulomb treatment (new key `coulomb`). */
#define MTG_COULOMB_ALLPAIRS 0 /* the reference: minimum image over all pairs, no cutoff
                                  (FunctorCalcForce.cpp:258-278,514-535) */
#define MTG_COULOMB_CUTOFF 1   /* truncated at coulomb_cutoff (new option) */
#define MTG_COULOMB_SHIFTED 2  /* shifted force, zero force and energy at coulomb_cutoff (new option):
                                  F = K qi qj (1/r^2 - 1/rc^2), U = K qi qj (1/r - 1/rc + (r - rc)/rc^2) */

/* Ensembles (SMolDynConfigStruct::Ensemble, MolDynConfigStruct.h:24).  NPT runs the reference's
 * MTK barostat and barostat chain (VelVerlet.cpp:57-71, 124-211, MDLoop.cpp:62-83) in every
 * precision mode; a batch refuses it.  The reference precision mode reproduces the reference's
 * arithmetic (barostat mass kT tauP^2, driven by sum F.r over wrapped positions).  The fp64 and
 * mixed modes drive the barostat with the pair virial (every pair's r_ij . F_ij plus the bonded
 * terms' virial), give it the MTK mass 3 (N + 1) kT tauP^2, and keep their Verlet list valid as
 * the box changes (the displacement test scales the build positions with the box; the cell grid
 * follows the box).  A box that shrinks until a cutoff reaches half its width ends the run with
 * MTG_E_UNSUPPORTED. */
#define MTG_NVT 0
#define MTG_NPT 1
#define MTG_NVE 2

/* One MDFF term: the kind code and up to four parameters, in the order listed above. */
typedef struct mtg_term {
    int32_t kind;
    int32_t reserved;
    double p[4];
} mtg_term;

/* System description.  Mirrors what CMDFFMatrices::prepareFFMatrices extracts from the state
 * (MDFFMatrices.cpp:181-536).  Atom types are numbered in first-appearance order of the atom IDs
 * (MolTwisterState.cpp:459-487).  Tables hold (x, -dU/dx, U) triples as produced by the MDFF
 * classes' calc1DForceProfile / calc1DPotentialProfile over [0.01, rc] (non-bonded, bonds) or
 * [0, 2 pi] (angles, dihedrals); pass NULL to have the library generate them from the terms
 * (the generator covers every kind except LJBuck and Class2, which then require tables). */
typedef struct mtg_system_desc {
    int32_t n_atoms;
    int32_t n_types;
    const double* r;            /* [n_atoms*3] positions */
    const double* p;            /* [n_atoms*3] momenta, or NULL for zero */
    const double* mass;         /* [n_atoms] */
    const double* charge;       /* [n_atoms] */
    const int32_t* type;        /* [n_atoms] 0..n_types-1 */
    const int32_t* mol;         /* [n_atoms] molecule index (-1 = none), or NULL */
    const uint8_t* mobile;      /* [n_atoms] 0/1, or NULL for all mobile */
    double box[3];              /* periodic box widths */
    /* Non-bonded terms per (row, col) type pair; row = type of the atom the force acts on. */
    const int32_t* nb_count;    /* [n_types*n_types] number of terms (<= MTG_MAX_FF_PER_PAIR) */
    const mtg_term* nb_terms;   /* [n_types*n_types*MTG_MAX_FF_PER_PAIR] */
    const float* nb_tables;     /* [n_types*n_types*MTG_MAX_FF_PER_PAIR*MTG_NPTS*3] or NULL */
    int32_t n_bond_types;
    const mtg_term* bond_terms; /* [n_bond_types] */
    const float* bond_tables;   /* [n_bond_types*MTG_NPTS*3] or NULL */
    int32_t n_angle_types;
    const mtg_term* angle_terms;
    const float* angle_tables;
    int32_t n_dih_types;
    const mtg_term* dih_terms;
    const float* dih_tables;
    /* Topology, as CMolTwisterStateTools::getAllMD{Bonds,Angles,Dihedrals}InSystem returns it
     * (MolTwisterStateTools.cpp:544-1209).  The order fixes the per-atom list order. */
    int32_t n_bonds;
    const int32_t* bonds;       /* [n_bonds*3]: atom i, atom j, bond type (-1 = skipped) */
    int32_t n_angles;
    const int32_t* angles;      /* [n_angles*4]: i, j (centre), k, angle type */
    int32_t n_dihedrals;
    const int32_t* dihedrals;   /* [n_dihedrals*5]: i, j, k, l, dihedral type */
} mtg_system_desc;

/* Run settings: the SMolDynConfigStruct fields the MD engine reads
 * (Config/MolDynConfigStruct.h:24-65, defaults Config/MolDynConfig.cpp:289-328) plus new keys. */
typedef struct mtg_config_desc {
    int32_t ensemble;           /* MTG_NVT / MTG_NPT / MTG_NVE */
    int32_t temperature_nh_len; /* temperaturenhlen (M, <= MTG_MAX_NH_CHAIN) */
    int32_t temperature_respa;  /* temperaturerespa */
    int32_t pressure_nh_len;    /* pressurenhlen */
    int32_t pressure_respa;     /* pressurerespa */
    int32_t precision;          /* MTG_PREC_* (new) */
    int32_t coulomb;            /* MTG_COULOMB_* (new) */
    int32_t clip_forces;        /* apply per-component clipping at cutoff_force (NVT/NVE) */
    double timestep;            /* fs */
    double temperature;         /* K */
    double temperature_relax;   /* fs */
    double pressure;            /* atm */
    double pressure_relax;      /* fs */
    double cutoff_radius;       /* A */
    double neigh_shell;         /* A, only sizes the cells (MDFFMatrices.cpp:45-58) */
    double cutoff_force;        /* cutoffforce */
    double scale12, scale13, scale14, scale1N;
    double coulomb_cutoff;      /* A, for MTG_COULOMB_CUTOFF (new) */
    double list_skin;           /* A, Verlet skin of the production neighbour list (new) */
    double opt_learning_rate;   /* optlearningrate */
    double opt_accuracy;        /* optaccuracy */
    int32_t opt_max_steps;      /* optmaxsteps */
    int32_t device;             /* CUDA device ordinal */
    int32_t lj_shift;           /* production modes, LJ at its cutoff (new): 0 truncated, 1 energy
                                   shifted to zero, 2 force shifted: F - F(rc), U - U(rc) + (r - rc) F(rc) */
    int32_t initial_max_neighbours; /* first capacity of the neighbour lists per atom (CNeighList::init,
                                   MDFFMatrices.cpp:93-99, which starts at 10); 0 = sized from the
                                   density.  Lists that overflow grow to need + 10 (reference) or need
                                   + 25 % (production) and the step or chunk is redone. */
} mtg_config_desc;

/* Thermostat/barostat state (CNHChain eta_/p_eta_, NHChain.h:55-61; CVelVerlet p_eps_, eps_,
 * VelVerlet.h:57-62).  Under NPT, mtg_set_state also sets the barostat momentum p_eps, the strain
 * eps (the box becomes (e^{3 eps})^{1/3} times the initial box) and the barostat chain NH_P_
 * (etaP/p_etaP, MP entries); box is output only (the current box). */
typedef struct mtg_thermo_state {
    int32_t M;
    int32_t reserved;
    double eta[MTG_MAX_NH_CHAIN];
    double p_eta[MTG_MAX_NH_CHAIN];
    double p_eps;
    double eps;
    int32_t MP;
    int32_t reserved2;
    double etaP[MTG_MAX_NH_CHAIN];
    double p_etaP[MTG_MAX_NH_CHAIN];
    double box[3];
} mtg_thermo_state;

/* Scalars of one output step (the info-line columns of MDLoop.cpp:388-403, in reduced units as
 * CSimulationBox returns them: T = sum p^2/m / 3N [kJ/mol], P [kJ/mol/A^3], V [A^3]). */
typedef struct mtg_output {
    int64_t step;               /* 0-based step index just completed */
    double T, P, V, U, K, E;
    const double* r;            /* [n_atoms*3] positions after the step (host, valid during the call) */
    const double* p;            /* [n_atoms*3] momenta after the step */
} mtg_output;

/* Output callback: return non-zero to stop the run early. */
typedef int (*mtg_output_cb)(const mtg_output* out, void* user);

typedef struct mtg_ctx mtg_ctx;

/* Library version (MTG_ABI_VERSION) and device name of ordinal `device`. */
int mtg_version(void);
int mtg_device_name(int device, char* buf, int buflen);

/* Tabulates one MDFF term on the host, as the term's calc1DForceProfile / calc1DPotentialProfile
 * do (MolTwisterMDFFNonBonded.cpp:126-172, MolTwisterMDFFBond.cpp:133-179,
 * MolTwisterMDFFAngle.cpp:210-257, MolTwisterMDFFDih.cpp:272-320): out[3*i .. 3*i+2] =
 * (x_i, -dU/dx, U) for x_i = x0 + i (x1 - x0)/(npts - 1).  No GPU is needed.  The reference calls
 * these with (0.01, rc) for non-bonded and bond terms and (0, 2 pi) for angles and dihedrals. */
int mtg_term_profile(const mtg_term* term, float x0, float x1, int npts, float* out);

/* Creates a context: validates the descriptors, uploads atoms, tables and topology, builds the
 * per-atom bonded lists (MDFFMatrices.cpp:384-520) and computes the initial forces.
 * Replaces CMDSimulator::run's setup half (MDSimulator.cpp:35-47, CSimulationBox ctor). */
int mtg_create(const mtg_system_desc* sys, const mtg_config_desc* cfg, mtg_ctx** out);
void mtg_destroy(mtg_ctx* ctx);
const char* mtg_last_error(const mtg_ctx* ctx);   /* ctx may be NULL (creation errors) */

/* Sets positions (NULL keeps), momenta (NULL keeps) and thermostat state (NULL keeps) and
 * recomputes forces.  Used to inject a seeded initial state (the reference draws it from rand(),
 * SimulationBox.cpp:98-133, NHChain.cpp:126-143). */
int mtg_set_state(mtg_ctx* ctx, const double* r, const double* p, const mtg_thermo_state* th);
int mtg_get_state(mtg_ctx* ctx, double* r, double* p, mtg_thermo_state* th);

/* Runs nsteps of the reference step sequence NH_P, NH_T, velocity-Verlet, NH_T, NH_P, pbcWrap
 * (MDLoop.cpp:128-133).  Every out_stride steps (step % out_stride == 0, as MDLoop.cpp:388) the
 * callback receives the output scalars and host copies of r and p; cb may be NULL.  out_stride
 * <= 0: no output steps (read the state with mtg_get_state). */
int mtg_run(mtg_ctx* ctx, int nsteps, int out_stride, mtg_output_cb cb, void* user);

/* Gradient-descent energy minimisation, CMDLoop::runOptimization (MDLoop.cpp:143-173). */
int mtg_optimize(mtg_ctx* ctx, double accuracy, int max_steps, int out_stride, mtg_output_cb cb, void* user);

/* Parity hooks. */
/* Forces and per-atom energies at the current positions, F = Fpi (no Ewald); any of the
 * pointers may be NULL.  U follows the reference bookkeeping (FunctorCalcForce.cpp:498-502,
 * 523-527, 562-566, 633-634, 700-701). */
int mtg_compute_forces(mtg_ctx* ctx, double* F, double* Fpi, double* U);
/* Cell list of the reference mode at the current positions: per-atom (ix,iy,iz), per-cell
 * first entry / count, and the cell-ordered atom list (FunctorGenCellList.cpp:49-142).  dims
 * receives the cell counts; ncells is the capacity of cell_first/cell_count. */
int mtg_get_cells(mtg_ctx* ctx, int32_t* dims, int32_t* ixyz, int32_t* cell_first, int32_t* cell_count,
                  int32_t ncells, int32_t* cell_list);
/* Full neighbour list of the reference mode at the current positions, in the reference order
 * (FunctorGenNeighList.cpp:72-151).  count[n]; list[n*max_neigh] when list != NULL;
 * *needed receives the largest count. */
int mtg_get_neighbors(mtg_ctx* ctx, int32_t max_neigh, int32_t* count, int32_t* list, int32_t* needed);

/* Timing/diagnostics of the last mtg_run: device milliseconds of the step loop, steps done,
 * neighbour-list rebuilds, and kernel launches per step. */
typedef struct mtg_run_stats {
    double device_ms;
    int64_t steps;
    int64_t list_builds;
    int64_t kernel_launches;
    int32_t graph_steps;        /* steps per captured CUDA graph (0 = not captured) */
    int32_t force_team;         /* lanes per atom chosen by the force-kernel autotuner */
    int32_t graph_form;         /* step-graph form: 0 plain capture, 1 list build under a conditional
                                   node, -1 not chosen yet (both are timed on the first chunks) */
} mtg_run_stats;
int mtg_get_run_stats(mtg_ctx* ctx, mtg_run_stats* st);

/* Initial momenta and Nose-Hoover / barostat state.
 *
 * MTG_INIT_REFERENCE: what CSimulationBox::initSystem draws (SimulationBox.cpp:53-96): chain
 * positions (NHChain.cpp:126-133), momenta uniform in [-1, 1) per component with 0 replaced by 1,
 * immobile atoms at rest, scaled to the temperature (SimulationBox.cpp:98-133), chain momenta
 * (NHChain.cpp:135-143) and the barostat momentum (VelVerlet.cpp:176-182), in that order, from the C
 * library's rand() seeded with `seed` (the reference draws in the CSimulationBox constructor,
 * before CMDLoop::runSimulation seeds rand() from the clock, MDLoop.cpp:118: a fresh MolTwister
 * process draws with seed 1).  As in the reference the momenta are scaled before the masses are
 * copied in, that is with a mass of 1 g/mol for every atom (Particle3D.cpp:25-27).
 * MTG_INIT_MAXWELL: seeded Maxwell-Boltzmann momenta with the real masses, the mobile atoms'
 * centre-of-mass momentum removed, scaled to sum p^2/m / 3N = kT; chain positions uniform in
 * [0, 1); chain and barostat momenta thermal (variance Q kT, W kT).  Not in the reference.
 *
 * mtg_draw_initial_state computes on the host only (p[3 n], *th) from the descriptors;
 * mtg_init_state draws for a context and sets the momenta and chain state (mtg_set_state), the
 * positions unchanged.  A batch returns MTG_E_UNSUPPORTED (set replicas' states one by one). */
#define MTG_INIT_REFERENCE 0
#define MTG_INIT_MAXWELL 1
int mtg_draw_initial_state(const mtg_system_desc* sys, const mtg_config_desc* cfg, uint32_t seed, int32_t mode, double* p,
                           mtg_thermo_state* th);
int mtg_init_state(mtg_ctx* ctx, uint32_t seed, int32_t mode);

/* Limit of every bounded device wait of this context (the thermostat chain's hand-overs between
 * warps), in polls of the flag; the default is 2^22.  A wait that runs out ends its kernel with
 * the values it has and the run returns MTG_E_TIMEOUT; the context stays usable after
 * mtg_set_state.  0 makes every wait give up at once (for testing the error path).  No counterpart
 * in the reference, which has no device waits. */
int mtg_set_wait_limit(mtg_ctx* ctx, int32_t polls);

/* Profiling hook (no counterpart in the reference, which only prints a per-step wall time,
 * MDLoop.cpp:434-456): runs `steps` un-captured steps with CUDA events around each phase on the
 * context's stream and returns the mean device milliseconds per step of
 * phase_ms[0] kick+drift, [1] list build (cell list / Verlet list; the early-exit kernels when no
 * rebuild is due), [2] force gather, [3] second kick + wrap + block sums (in the reference and FP64
 * modes also the system totals and the thermostat chain, which run in that kernel's last block),
 * [4] mixed mode's step-end kernel (system totals, thermostat chain, output record; 0 otherwise).
 * phase_ms holds 5 values.  The state advances by `steps` steps exactly as mtg_run would advance
 * it. */
int mtg_profile_phases(mtg_ctx* ctx, int steps, double* phase_ms);

/* ---- Force-field parameters and gradients (no counterpart in the reference, which has no
 * derivatives) ----
 *
 * A parameter is one scalar of the MDFF terms: the epsilon or sigma of the LJ term of a type pair
 * (index = row * n_types + col; both orders of the pair follow), a direction in charge space
 * (q_i = theta * dq[i] for every atom with dq[i] != 0, e.g. dq = 1 on O and -1/2 on H makes theta
 * the oxygen charge of a neutral water), or k / r0 of a harmonic bond type, or k / theta0 [deg] of a
 * harmonic angle type (index = term type).  Gradients use the analytic terms of the fp64 / mixed
 * modes, in FP64 arithmetic (forward-mode dual numbers for the force tangents). */
#define MTG_P_LJ_EPS 1
#define MTG_P_LJ_SIGMA 2
#define MTG_P_CHARGE 3
#define MTG_P_BOND_K 4
#define MTG_P_BOND_R0 5
#define MTG_P_ANGLE_K 6
#define MTG_P_ANGLE_THETA0 7
typedef struct mtg_param {
    int32_t kind;
    int32_t index;
    const double* dq;          /* MTG_P_CHARGE: [n_atoms] direction */
} mtg_param;

int mtg_get_params(mtg_ctx* ctx, int32_t nparams, const mtg_param* params, double* values);
/* Changes the parameters and recomputes the forces (fp64 / mixed modes). */
int mtg_set_params(mtg_ctx* ctx, int32_t nparams, const mtg_param* params, const double* values);
/* Total potential energy at the current positions and its derivatives d U / d theta_k. */
int mtg_energy_grad(mtg_ctx* ctx, int32_t nparams, const mtg_param* params, double* U, double* grad);
/* A batch's per-replica energies U[nrep] and derivatives grad[r * nparams + k] = d U_r / d theta_k
 * of the shared force-field parameters, from one force-tangent pass per parameter over all
 * replicas and deterministic per-replica sums.  The single-system form above refuses batches. */
int mtg_batch_energy_grad(mtg_ctx* ctx, int32_t nparams, const mtg_param* params, double* U, double* grad);

/* Short-trajectory loss: from the current state, `nsteps` plain velocity-Verlet steps (NVE, no
 * force clipping, whatever the context's ensemble), and the squared deviation
 *     L = sum_b (gbar_b - target_b)^2
 * of the Gaussian-smeared pair correlation of types type_a and type_b averaged over the positions
 * after each step: g_b = V / (N_pairs 4 pi x_b^2) sum_pairs K(r_ij - x_b), x_b = (b + 1/2) rmax /
 * nbins, K the unit-area Gaussian of standard deviation `width` taken where |r_ij - x_b| <= 8 width
 * (pairs of the Verlet list, which must reach rmax + 8 width; bonded exclusions are not counted).  The gradient dL/dtheta comes from the discrete adjoint of the
 * velocity-Verlet recursion, run backwards with states stored every checkpoint_every steps and the
 * positions in between recomputed (memory: (nsteps / checkpoint_every + checkpoint_every) position
 * sets).  With grad == NULL (or nparams == 0) only the loss is evaluated.  The context's state is
 * unchanged on return. */
typedef struct mtg_loss_desc {
    int32_t nsteps;
    int32_t checkpoint_every;
    int32_t type_a, type_b;
    int32_t nbins;
    int32_t reserved;
    double rmax, width;
    const double* target;      /* [nbins] */
} mtg_loss_desc;
int mtg_loss_grad(mtg_ctx* ctx, const mtg_loss_desc* loss_desc, int32_t nparams, const mtg_param* params,
                  double* loss, double* grad, double* rdf /* [nbins] or NULL: gbar */);

/* Pair-distance histogram of `moldyn`'s sibling analysis command `calculate paircorrelation`
 * (Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.cpp:182-215) for the current positions: every
 * ordered pair (i of type_a, j of type_b, including i == j when the types are equal), distance
 * across the periodic box, pairs closer than ignore_below skipped (the command's `ignoredistbelow`,
 * -1 for none), bin int((R - rmin) / (rmax - rmin) * nbins).  The counts are added to profile[nbins]
 * so that successive calls accumulate frames; the command's normalisation to g(r) is a host step
 * (moltwister_gb300.analysis.PairCorrelation).  nbins <= 8192. */
int mtg_pair_histogram(mtg_ctx* ctx, int32_t type_a, int32_t type_b, int32_t nbins, double rmin, double rmax,
                       double ignore_below, int64_t* profile);

/* Trajectory files of the output step, byte for byte as the reference writes them.
 * mtg_dcd_append creates the file with its header (num_steps / out_stride sets, time step in fs)
 * if it does not exist, then appends one record: the box truncated to integers as
 * CMDLoop::appendToDCDFile passes it (MDLoop.cpp:248-258, Utilities/DCDFile.cpp:670-729), FP32
 * coordinates.  mtg_xyz_append appends one frame as CMDLoop::appendToXYZFile (MDLoop.cpp:229-246).
 * Host-only; r is the host copy an mtg_run callback receives. */
int mtg_dcd_append(const char* path, int32_t n_atoms, const double* r, const double box[3], int32_t num_steps,
                   int32_t out_stride, double timestep_fs);
int mtg_xyz_append(const char* path, int32_t n_atoms, const double* r, const char* const* ids, int32_t step);

/* ---- Batches of independent replicas (no counterpart in the reference, which runs one system
 * per `moldyn run`) ----
 *
 * mtg_batch_create merges nrep systems that share one force field (same n_types, non-bonded terms
 * per type pair and bonded term types; analytic terms only) into one context whose kernels advance
 * every replica per launch: atoms are concatenated (replica r owns atoms offsets[r] ..
 * offsets[r+1]-1), each replica keeps its own box, cell grid, temperature (temperatures[r] K, or
 * cfg->temperature when NULL), pair cutoff (cutoffs[r] A for LJ and Coulomb, at most
 * cfg->cutoff_radius, or the shared cutoffs when NULL: small boxes need shorter ones for the
 * minimum image), Nose-Hoover chain and energies.  cfg is shared (fp64 or mixed
 * precision, NVT or NVE).  A replica's trajectory equals, bit for bit, the trajectory of the same
 * system run alone in mixed precision.  The returned context works with mtg_run, mtg_get_state /
 * mtg_set_state (positions and momenta of all replicas, without the chain argument),
 * mtg_compute_forces, mtg_get_run_stats and mtg_destroy; mtg_run's callback receives the ensemble's
 * totals (U, K, E and V summed, T over all atoms, P averaged) and mtg_batch_get_records gives the
 * per-replica values of the same output step. */
int mtg_batch_create(const mtg_system_desc* const* systems, int32_t nrep, const mtg_config_desc* cfg,
                     const double* temperatures, const double* cutoffs, mtg_ctx** out);
int mtg_batch_info(mtg_ctx* ctx, int32_t* nrep, int32_t* offsets /* nrep + 1 */);
/* rec[6 r + 0..5] = T, P, V, U, K, E of replica r at the last output step of mtg_run */
int mtg_batch_get_records(mtg_ctx* ctx, double* rec);
int mtg_batch_set_thermo(mtg_ctx* ctx, int32_t rep, const mtg_thermo_state* th);
int mtg_batch_get_thermo(mtg_ctx* ctx, int32_t rep, mtg_thermo_state* th);

/* ---- No-allocation neighbour list (no counterpart in the reference) ----
 *
 * The reference has no such entry point: its neighbour list is built inside CMDFFMatrices, which
 * owns its device vectors (MDFFMatrices.cpp:163-178).  This one serves callers that hold atom
 * positions in device memory they manage themselves and must not allocate: an analysis pass
 * (pair correlation, clustering) running next to a live simulation, where cudaMalloc/cudaFree
 * would synchronise the device and stall the simulation's streams, or a host framework whose
 * caching allocator already holds the GPU's memory.  mtg_create allocates, so those callers use
 * this instead.
 *
 * It computes the same reference-order cell assignment and full neighbour list as
 * mtg_get_neighbors (FunctorGenCellList.cpp:49-142, FunctorGenNeighList.cpp:72-151) for the
 * positions d_r[3n] (FP64, device memory of the current device) in a box centred at the origin,
 * with cells floor(float(L)/(cutoff + shell)) per axis (MDFFMatrices.cpp:56-58).  Outputs, in
 * device memory the caller owns: d_count[n] (full neighbour count of each atom, also when it
 * exceeds max_neigh) and d_list[n * max_neigh] (the first max_neigh neighbours of each atom; may
 * be NULL when max_neigh is 0).
 *
 * Working memory is one file-scope device array of MTG_NOALLOC_SCRATCH_BYTES per device; the call
 * needs 16 bytes per atom plus 12 bytes per cell (each part rounded up to 256 bytes) plus 256
 * bytes, and returns MTG_E_INVALID without launching anything when that exceeds the array
 * (about a million atoms in a million cells; larger systems use mtg_create).  It performs no
 * device allocation and calls no allocating library function.
 *
 * `stream` is a cudaStream_t (NULL = the legacy default stream).  With needed == NULL the call
 * only enqueues work and returns; with needed != NULL it waits for the stream and stores in
 * *needed the largest neighbour count when some atom has more than max_neigh neighbours (its list
 * in d_list is truncated; d_count still holds the full counts), or 0 when every list fits.
 *
 * Limits the caller must respect: the scratch array is shared by every call on a device, so calls
 * whose work overlaps in time (other streams, other host threads, or a second call enqueued on
 * another stream before the first finished) race on it and must be serialised by the caller;
 * calls enqueued one after another on the same stream are safe.  Every call looks up the array's
 * address in the current context (cudaGetSymbolAddress), so a device reset or a caller-made
 * context between calls is followed; the first call on each device also loads the module there,
 * so make that first call before any stream capture begins on that device.  Errors are reported
 * through mtg_last_error(NULL) of the calling thread. */
#define MTG_NOALLOC_SCRATCH_BYTES (32u << 20)
int mtg_neighbors_noalloc(const double* d_r, int32_t n, const double box[3], double cutoff, double shell,
                          int32_t max_neigh, int32_t* d_count, int32_t* d_list, int32_t* needed, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MTGPU_H */
