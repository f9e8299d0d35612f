"""GPU parity: libmtgpu.so through its C ABI against the reference's own outputs (tests/golden/)
and against the CPU oracle.

Tolerances (stated per test):
  - cell assignment and neighbour lists: bit-exact;
  - reference-mode forces: 1e-12 relative to the largest force (FP64 with the reference's order;
    only libm acos on the angle/dihedral paths may differ in the last bit); per-atom energies
    (FP32 sums) 1e-5 relative;
  - reference-mode 100-step trajectories: positions and momenta within 1e-8 relative to their
    scale, energies within 1e-8 relative (the thermostat's kinetic sum is reduced in a different
    order on the GPU, so the trajectories agree to rounding, not bit for bit); under NPT also the
    barostat momentum p_eps and the volume within 1e-8 relative;
  - analytic FP64 mode vs the FP64 oracle: 1e-10 relative RMS;
  - mixed mode (FP32 arithmetic, int64 fixed-point sums) vs the FP64 oracle: 1e-5 relative RMS
    force error, the target the mixed mode is specified to.
"""
import numpy as np
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu

CASES = G.names()


@pytest.fixture(scope="module", autouse=True)
def built():
    from moltwister_gb300.build import build
    build()


def engine(s, cfg, **kw):
    from moltwister_gb300.engine import Engine
    return Engine(s, cfg, **kw)


def golden_tables(s, d):
    from oracle.oracle import reference_nb_layout
    T = len(s.type_names())
    return {"nb": reference_nb_layout(d["nb_table"], T), "bond": d["bond_table"].reshape(-1, 1000, 3),
            "angle": d["angle_table"].reshape(-1, 1000, 3), "dih": d["dih_table"].reshape(-1, 1000, 3)}


@pytest.mark.parametrize("name", CASES)
def test_cells_bit_exact(name):
    s, cfg, d = G.load(name)
    e = engine(s, cfg, tables=golden_tables(s, d))
    dims, ixyz, first, count, lst = e.cells()
    assert tuple(dims) == tuple(d["cell_dims"])
    assert np.array_equal(ixyz, d["atom_cell"])
    assert np.array_equal(first, d["cell_ptr"][:, 0])
    assert np.array_equal(count, d["cell_ptr"][:, 1])
    assert np.array_equal(lst, d["cell_list"])


@pytest.mark.parametrize("name", CASES)
def test_neighbours_bit_exact(name):
    s, cfg, d = G.load(name)
    e = engine(s, cfg, tables=golden_tables(s, d))
    cnt, lst = e.neighbors()
    assert G.neighbours_match(d, cnt, lst)


@pytest.mark.parametrize("name", CASES)
def test_reference_forces(name):
    s, cfg, d = G.load(name)
    e = engine(s, cfg, tables=golden_tables(s, d))
    F, U = e.forces()
    scale = np.abs(d["F"]).max()
    assert np.abs(F - d["F"]).max() <= 1e-12 * scale
    assert np.allclose(U, d["U"].astype(np.float64), rtol=1e-5, atol=1e-5 * np.abs(d["U"]).max())


@pytest.mark.parametrize("n_mol", [216, 1000])
def test_reference_coulomb_bit_exact(n_mol):
    """Charged water with its angle terms taken out (no acos on any path) and every eleventh atom
    held fixed: reference-mode forces and per-atom energies equal the oracle's reference-order
    restatement bit for bit.  This pins the order of each atom's sum (bonds, then short-range
    pairs in neighbour-list order, then the all-pairs Coulomb terms in ascending j,
    FunctorCalcForce.cpp:159-281, including the tail tiles of 648 atoms) and the FP64 square
    root, division and minimum image of every one of the 0.4 and 9 million pairs."""
    from moltwister_gb300 import workloads as W
    from oracle import oracle as O
    s, cfg = W.water(n_mol=n_mol, L=W.water_box_length(n_mol), seed=14, rc=6.0)
    s.angles = np.zeros((0, 4), np.int32)
    s.angle_terms = []
    s.mobile[5::11] = False
    assert cfg.precision == "reference" and cfg.coulomb == "allpairs"
    orc = O.Oracle(s, cfg)
    t = orc.tabs
    e = engine(s, cfg, tables={"nb": t["nb"], "bond": t["bond"], "angle": t["angle"], "dih": t["dih"]})
    F, U = e.forces()
    Fo, Uo = orc.forces_ref()
    assert np.abs(F).max() > 0 and np.abs(Uo).max() > 0
    assert np.array_equal(F, Fo), np.abs(F - Fo).max()
    assert np.array_equal(U, Uo.astype(np.float64)), np.abs(U - Uo).max()


@pytest.mark.parametrize("name", CASES)
def test_reference_trajectory(name):
    s, cfg, d = G.load(name)
    e = engine(s, cfg, tables=golden_tables(s, d))
    stride, steps = int(d["stride"]), int(d["steps"])
    r_scale = float(np.abs(d["traj_r"]).max())
    p_scale = float(np.abs(d["traj_p"]).max())
    for rec in range(1, d["traj_r"].shape[0]):
        n = stride if rec * stride <= steps else steps - (rec - 1) * stride
        out = e.run(n, out_stride=n - 1 if n > 1 else 1)
        r, p, _ = e.get_state()
        assert np.abs(r - d["traj_r"][rec]).max() <= 1e-8 * r_scale, rec
        assert np.abs(p - d["traj_p"][rec]).max() <= 1e-8 * p_scale, rec
        last = out[-1]
        U, K, T, P, V = d["traj_scalars"][rec, 1:6]
        assert abs(last.U - U) <= 1e-8 * max(1.0, abs(U))
        assert abs(last.K - K) <= 1e-8 * max(1.0, abs(K))
        assert abs(last.T - T) <= 1e-8 * max(1.0, abs(T))
        # NPT: V = V0 exp(3 eps) follows the barostat, which sees the same rounding differences
        assert abs(last.V - V) <= (1e-8 if cfg.ensemble == "NPT" else 1e-12) * V
        if cfg.ensemble == "NPT":
            _, _, th = e.get_state()
            pe = float(d["traj_peps"][rec])
            assert abs(th.p_eps - pe) <= 1e-8 * max(1.0, abs(pe)), (rec, th.p_eps, pe)
            assert np.allclose(th.box, V ** (1 / 3) * s.box / np.prod(s.box) ** (1 / 3), rtol=1e-8)


def analytic_case(coulomb="cutoff"):
    """Water in a >=3-cell box with cutoff Coulomb; a jittered copy of the golden input."""
    s, cfg, d = G.load("water648_nvt")
    s.r = s.r + np.random.default_rng(7).uniform(-0.02, 0.02, s.r.shape)
    cfg.coulomb = coulomb
    cfg.coulombcutoff = cfg.cutoffradius
    return s, cfg


@pytest.mark.parametrize("coulomb", ["cutoff", "shifted"])
def test_fp64_mode_matches_fp64_oracle(coulomb):
    from oracle import oracle as O
    s, cfg = analytic_case(coulomb)
    cfg.precision = "fp64"
    F, U = engine(s, cfg).forces()
    Fo, Uo = O.Oracle(s, cfg).forces_fp64()
    rel = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    assert rel < 1e-10, rel
    assert abs(U.sum() - Uo.sum()) < 1e-9 * abs(Uo.sum())


@pytest.mark.parametrize("coulomb", ["cutoff", "shifted"])
def test_mixed_mode_force_error(coulomb):
    from oracle import oracle as O
    s, cfg = analytic_case(coulomb)
    cfg.precision = "mixed"
    F, U = engine(s, cfg).forces()
    Fo, Uo = O.Oracle(s, cfg).forces_fp64()
    rel = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    assert rel < 1e-5, rel
    assert abs(U.sum() - Uo.sum()) < 1e-5 * abs(Uo.sum())


def test_mixed_mode_bit_reproducible():
    """Fixed-point accumulation: two evaluations, and a run repeated from the same state, agree
    bit for bit."""
    s, cfg = analytic_case()
    cfg.precision = "mixed"
    e1 = engine(s, cfg)
    F1, _ = e1.forces()
    F2, _ = e1.forces()
    assert np.array_equal(F1, F2)
    e1.run(50)
    r1, p1, _ = e1.get_state()
    e2 = engine(s, cfg)
    e2.run(50)
    r2, p2, _ = e2.get_state()
    assert np.array_equal(r1, r2) and np.array_equal(p1, p2)


def test_step_graph_form_and_team_do_not_change_results():
    """The run picks its step-graph form from four alternating timed chunks (conditional, plain,
    conditional, plain) and re-times the force gather's team size at its first run; the statistics
    report both.  A 100-step run in those chunks and one in chunks too short to time (plain form
    throughout) reach the same state bit for bit: forms, team sizes and output steps do not change
    the arithmetic.  (Splitting a run into several runs does round differently: each run ends by
    applying the pending thermostat scale to the momenta.)"""
    s, cfg = analytic_case()
    cfg.precision = "mixed"
    e1 = engine(s, cfg)
    e1.run(100, out_stride=20)          # chunks of 20 steps: four timed, then the chosen form
    st = e1.stats()
    assert st["graph_form"] in (0, 1), st
    assert st["force_team"] in (8, 16, 32), st
    r1, p1, _ = e1.get_state()
    e2 = engine(s, cfg)
    e2.run(100, out_stride=10)          # chunks of 10 steps: below the tuning length
    r2, p2, _ = e2.get_state()
    assert np.array_equal(r1, r2) and np.array_equal(p1, p2)


def test_mixed_state_round_trip():
    """Mixed mode keeps positions and momenta as double-float pairs and box fractions on the
    device; the host reads and writes FP64.  Reading the state changes nothing (50 + read + 50
    steps is bit-identical to 100 steps), and writing it back changes it by at most the FP64
    rounding of a double-float whose low part lies more than 53 bits below its high part: NVE,
    the state read and written back after 50 steps, then 50 more steps within 1e-10 of the
    straight run (the difference of ~1e-16 grows with the dynamics' divergence)."""
    from moltwister_gb300 import workloads as W
    s, cfg = W.kob_andersen(ncell=6, seed=9)
    e1 = engine(s, cfg)
    e1.run(100)
    r1, p1, _ = e1.get_state()
    e3 = engine(s, cfg)
    e3.run(50)
    e3.get_state()
    e3.run(50)
    r3, p3, _ = e3.get_state()
    assert np.array_equal(r1, r3) and np.array_equal(p1, p3)
    e2 = engine(s, cfg)
    e2.run(50)
    r, p, _ = e2.get_state()
    e2.set_state(r=r, p=p)
    r0, p0, _ = e2.get_state()
    assert np.array_equal(r, r0) and np.array_equal(p, p0)
    e2.run(50)
    r2, p2, _ = e2.get_state()
    assert np.abs(r1 - r2).max() < 1e-10 * np.abs(r1).max()
    assert np.abs(p1 - p2).max() < 1e-10 * np.abs(p1).max()


def test_mixed_integrator_tracks_fp64_on_a_regular_orbit():
    """Two bonded atoms (harmonic bond, no other interaction) oscillate on a regular orbit, so
    trajectories do not diverge: after 4,000 NVE steps (77 periods) the double-float integrator
    with FP32 forces agrees with the FP64 path to 2e-5 in positions (A) and momenta (relative to
    their amplitude).  The FP32 force's relative error of ~1e-7 shifts the frequency by as much,
    a phase error of ~5e-5 rad after 77 periods on a 0.15 A amplitude; an integrator error
    (a wrong factor in a kick or the drift) would show at the 1e-2 level."""
    from moltwister_gb300.system import BondTerm, MDConfig, MDSystem
    r = np.array([[0.0, 0.0, 0.0], [1.15, 0.1, -0.05]])
    s = MDSystem(box=np.array([20.0, 20.0, 20.0]), ids=["A", "B"], r=r, q=np.zeros(2), m=np.array([12.0, 16.0]),
                 mobile=np.ones(2, bool), bond_terms=[BondTerm("A", "B", "Harm", (2000.0, 1.0))],
                 bonds=np.array([[0, 1, 0]], np.int32))
    s.p = np.array([[0.5, -0.2, 0.1], [-0.5, 0.2, -0.1]])
    out = {}
    for prec in ("fp64", "mixed"):
        cfg = MDConfig(timestep=0.5, ensemble="NVE", cutoffradius=5.0, neighshell=0.5, listskin=0.5,
                       precision=prec, coulomb="cutoff", coulombcutoff=5.0, clipforces=False)
        e = engine(s, cfg)
        e.run(4000)
        out[prec] = e.get_state()[:2]
    (r64, p64), (rm, pm) = out["fp64"], out["mixed"]
    assert np.abs(rm - r64).max() < 2e-5, np.abs(rm - r64).max()
    assert np.abs(pm - p64).max() < 2e-5 * np.abs(p64).max(), np.abs(pm - p64).max()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_production_chain_terms(prec):
    """Bonds (Harm, Morse), angles, dihedrals (Harm), Buckingham + LJ, immobile atoms."""
    from oracle import oracle as O
    s, cfg, d = G.load("chains108_nvt")
    s.r = s.r + np.random.default_rng(3).uniform(-0.03, 0.03, s.r.shape)
    cfg.precision = prec
    cfg.coulomb = "cutoff"
    cfg.coulombcutoff = cfg.cutoffradius
    F, U = engine(s, cfg).forces()
    Fo, Uo = O.Oracle(s, cfg).forces_fp64()
    rel = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    assert rel < (1e-10 if prec == "fp64" else 2e-5), rel


def test_optimize_reference_matches_oracle():
    """Gradient descent in reference mode (CMDLoop::runOptimization, SimulationBox.cpp:197-208)
    follows the reference's own energy sequence, which is not monotonic on this input."""
    from oracle import oracle as O
    s, cfg, d = G.load("water648_nvt")
    cfg.optlearningrate = 1e-5
    e = engine(s, cfg)
    recs = e.optimize(8, out_stride=1)
    orc = O.Oracle(s, cfg)
    r = orc.r.copy()
    ref = []
    for _ in range(8):
        orc.set_positions(r)
        F, u = orc.forces_ref()
        ref.append(u.astype(np.float64).sum())
        r = r + F * cfg.optlearningrate
    got = np.array([x.U for x in recs])
    assert np.allclose(got, ref, rtol=1e-9, atol=1e-6), (got, ref)


def test_optimize_mixed_lowers_energy():
    s, cfg, d = G.load("water648_nvt")
    cfg.precision = "mixed"
    cfg.coulomb = "shifted"
    cfg.coulombcutoff = cfg.cutoffradius
    cfg.optlearningrate = 1e-5
    recs = engine(s, cfg).optimize(30, out_stride=1)
    U = [r.U for r in recs]
    assert len(U) == 30
    assert all(np.diff(U) < 0), U[:5]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_kob_andersen_per_pair_cutoffs(prec):
    """Binary LJ mixture with a cutoff of 2.5 sigma_ab per pair and energies shifted to zero at
    the cutoffs (new options of the production modes) against the FP64 oracle."""
    from oracle import oracle as O
    from moltwister_gb300 import workloads as W
    s, cfg = W.kob_andersen(ncell=6, seed=5)
    cfg.precision = prec
    F, U = engine(s, cfg).forces()
    Fo, Uo = O.Oracle(s, cfg).forces_fp64()
    rel = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    assert rel < (1e-10 if prec == "fp64" else 1e-5), rel
    assert abs(U.sum() - Uo.sum()) < (1e-9 if prec == "fp64" else 1e-5) * abs(Uo.sum())


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_nve_conserves_energy(prec):
    """NVE on a 16,384-atom Kob-Andersen mixture with force-shifted LJ (continuous forces): after
    4,000 steps of equilibration the linear drift of the total energy over 8,000 steps (4 ps) stays
    below 2e-2 kT per atom per ns in FP64 and in mixed precision (double-float integration, FP32
    pair forces).  The fitted slope of so short a window carries the velocity-Verlet energy
    fluctuation as noise, about 5e-3 kT per atom per ns here (from the standard error measured on
    131,072 atoms over 40 ps, scaled by N^-1/2 and window^-3/2), so the bound catches a broken
    integrator, not the 1e-4 target: bench_drift measures that (both precisions drift by
    -1.2e-4 +- 0.5e-4 on 131,072 atoms over 40 ps)."""
    from moltwister_gb300 import workloads as W
    s, cfg = W.kob_andersen(ncell=16, seed=6)
    cfg.precision = prec
    cfg.ljshift = 2
    e = engine(s, cfg)
    e.optimize(200)
    e.run(4000)                                        # equilibrate the relaxed lattice start
    recs = e.run(8000, out_stride=100)
    t_ns = np.array([r.step for r in recs], float) * cfg.timestep * 1e-6
    E = np.array([r.U + r.K for r in recs])
    kT = cfg.temperature / 120.272
    slope = np.polyfit(t_ns, E, 1)[0]
    drift = abs(slope) / (s.n * kT)
    assert drift < 2e-2, drift


def test_production_chain_stays_finite_on_large_systems():
    """An 11,681-atom argon replica at 96 K whose chain diverges (NaN after ~350 steps) with the
    reference's Suzuki-Yoshida weights, CMt::exp and p_eta[0] clamp stays finite and near its
    temperature with the production modes' chain integrator."""
    from moltwister_gb300 import workloads as W
    from moltwister_gb300.system import MDConfig
    spec = W.replica_spec(64, seed=5)
    kind, n, T, seed = spec[51]
    s, rc = W.make_replica(kind, n, T, seed)
    cfg = MDConfig(timestep=0.5, ensemble="NVT", temperature=T, temperaturerelax=20.0, cutoffradius=rc,
                   neighshell=1.0, coulomb="shifted", coulombcutoff=rc, listskin=1.0, precision="mixed")
    e = engine(s, cfg)
    recs = e.run(3000, out_stride=100)
    T_K = np.array([r.T for r in recs]) * 120.272
    assert np.all(np.isfinite(T_K))
    assert abs(T_K[-10:].mean() - T) < 0.15 * T, (T_K[-10:], T)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_force_shifted_lj(prec):
    """Force-shifted LJ (ljshift = 2, a new option) against the FP64 oracle."""
    from oracle import oracle as O
    s, cfg = analytic_case("shifted")
    cfg.precision = prec
    cfg.ljshift = 2
    F, U = engine(s, cfg).forces()
    Fo, Uo = O.Oracle(s, cfg).forces_fp64()
    rel = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    assert rel < (1e-10 if prec == "fp64" else 1e-5), rel
    assert abs(U.sum() - Uo.sum()) < (1e-9 if prec == "fp64" else 1e-5) * abs(Uo.sum())
