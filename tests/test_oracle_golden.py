"""The CPU oracle (oracle/mdoracle.c) against the reference's own outputs (tests/golden/).

Everything here is bit-exact: the oracle restates the reference's arithmetic in the same order
without fused multiply-adds, and the fixtures come from the reference built the same way."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

CASES = G.names()


@pytest.mark.parametrize("name", CASES)
def test_tables_bit_exact(name):
    s, cfg, d = G.load(name)
    t = O.tables(s, cfg)
    T = len(s.type_names())
    assert np.array_equal(O.reference_nb_layout(d["nb_table"], T).view(np.uint32), t["nb"].view(np.uint32))
    assert np.array_equal(d["nb_count"].reshape(T, T), t["nb_count"])
    for key, ref in (("bond", "bond_table"), ("angle", "angle_table"), ("dih", "dih_table")):
        assert np.array_equal(d[ref].reshape(-1, 1000, 3).view(np.uint32), t[key].view(np.uint32)), key


@pytest.mark.parametrize("name", CASES)
def test_cells_and_neighbours_bit_exact(name):
    s, cfg, d = G.load(name)
    orc = O.Oracle(s, cfg)
    assert tuple(d["cell_dims"]) == orc.cells
    ac, cp, cl = orc.cell_list()
    assert np.array_equal(ac, d["atom_cell"])
    assert np.array_equal(cp, d["cell_ptr"])
    assert np.array_equal(cl, d["cell_list"])
    cnt, lst = orc.neigh_list()
    assert G.neighbours_match(d, cnt, lst)
    m = d["neigh_list"].shape[1] if "neigh_list" in d else int(d["neigh_max"])
    assert m == cnt.max()


@pytest.mark.parametrize("name", CASES)
def test_forces_bit_exact(name):
    s, cfg, d = G.load(name)
    F, U = O.Oracle(s, cfg).forces_ref()
    assert np.array_equal(F, d["F"])
    assert np.array_equal(U, d["U"])


@pytest.mark.parametrize("name", CASES)
def test_trajectory_bit_exact(name):
    s, cfg, d = G.load(name)
    if "prefix_steps" in d:
        # the full-size cases (4,000-atom argon, 9,000-atom water): the oracle replays the reference's short prefix run (the
        # 100-step trajectory is checked against the GPU, which the oracle is pinned to here)
        k = int(d["prefix_steps"])
        o = O.Oracle(s, cfg).run_ref(k, k)
        assert np.array_equal(o["r"][-1], d["prefix_r"])
        assert np.array_equal(o["p"][-1], d["prefix_p"])
        assert np.array_equal(o["scal"][-1], d["prefix_scalars"][1:6])
        return
    o = O.Oracle(s, cfg).run_ref(int(d["steps"]), int(d["stride"]))
    assert np.array_equal(o["r"], d["traj_r"])
    assert np.array_equal(o["p"], d["traj_p"])
    assert np.array_equal(o["F"], d["traj_F"])
    assert np.array_equal(o["scal"], d["traj_scalars"][:, 1:6])
    M = cfg.temperaturenhlen
    if cfg.ensemble in ("NVT", "NPT"):
        assert np.array_equal(o["eta"], d["traj_nhT"][-1, 0, :M])
        assert np.array_equal(o["peta"], d["traj_nhT"][-1, 1, :M])
    if cfg.ensemble == "NPT":
        MP = cfg.pressurenhlen
        assert o["p_eps"] == d["traj_peps"][-1]
        assert np.array_equal(o["etaP"], d["traj_nhP"][-1, 0, :MP])
        assert np.array_equal(o["petaP"], d["traj_nhP"][-1, 1, :MP])


def test_npt_volume_changes():
    """The NPT golden cases really move the box (VelVerlet.cpp:57-71, getSimBox :198-211)."""
    for name in ("argon500_npt", "water648_npt"):
        s, cfg, d = G.load(name)
        V = d["traj_scalars"][:, 5]
        assert np.all(np.isfinite(V)) and abs(V[-1] - V[0]) > 1e-3 * V[0], (name, V)


def test_two_cells_duplicate_neighbours():
    """With fewer than 3 cells per axis the reference scans wrapped cells twice and lists the same
    neighbour more than once (FunctorGenNeighList.cpp:79-99); the oracle reproduces it."""
    s, cfg, d = G.load("argon256_2cells")
    assert tuple(d["cell_dims"]) == (2, 2, 2)
    lst, cnt = d["neigh_list"], d["neigh_count"]
    dup = sum(len(lst[k, :cnt[k]]) - len(set(lst[k, :cnt[k]].tolist())) for k in range(s.n))
    assert dup > 0


def test_analytic_forces_match_energy_gradient():
    """The FP64 analytic oracle: forces are minus the gradient of its total energy (central
    differences on a jittered chain system with every analytic term kind)."""
    from moltwister_gb300 import workloads as W
    s, cfg = W.chains(n_chain=8, L=16.0, seed=3)
    s.r = s.r + np.random.default_rng(0).uniform(-0.05, 0.05, s.r.shape)
    orc = O.Oracle(s, cfg)
    F, _ = orc.forces_fp64()
    r0 = orc.r.copy()
    h = 1e-6
    for k in (0, 1, 5, 13, 22):
        for a in range(3):
            rp = r0.copy(); rp[k, a] += h
            rm = r0.copy(); rm[k, a] -= h
            up = orc.set_positions(rp).forces_fp64()[1].sum()
            um = orc.set_positions(rm).forces_fp64()[1].sum()
            assert abs(-(up - um) / (2 * h) - F[k, a]) < 1e-5 * max(1.0, abs(F[k, a]))
    orc.set_positions(r0)


def test_analytic_close_to_tables_where_reference_is_valid():
    """Analytic FP64 vs the reference tables on a >=3-cell water case: they differ only by the
    table interpolation error (Coulomb is analytic in both)."""
    s, cfg, d = G.load("water648_nvt")
    F, _ = O.Oracle(s, cfg).forces_fp64()
    rel = np.sqrt(((F - d["F"]) ** 2).sum() / (d["F"] ** 2).sum())
    assert rel < 1e-4


def test_force_shifted_lj_forces_are_energy_gradient():
    """Oracle, ljshift = 2: the LJ force and energy are continuous at the cutoff and F = -grad U."""
    from moltwister_gb300 import workloads as W
    s, cfg = W.kob_andersen(ncell=3, seed=5, jitter=0.1)
    cfg.precision = "fp64"
    cfg.ljshift = 2
    orc = O.Oracle(s, cfg)
    F, U = orc.forces_fp64()
    h = 1e-6
    for k, a in [(0, 0), (5, 1), (17, 2)]:
        r = s.r.copy(); r[k, a] += h; orc.set_positions(r); Up = orc.forces_fp64()[1].sum()
        r = s.r.copy(); r[k, a] -= h; orc.set_positions(r); Um = orc.forces_fp64()[1].sum()
        assert abs(F[k, a] + (Up - Um) / (2 * h)) < 1e-6 * max(1.0, abs(F[k, a]))
