"""Batches of replicas (mtg_batch_create): argon and water replicas of different sizes and
temperatures advanced together must each follow, bit for bit, the trajectory of the same system
run alone in mixed precision (forces are exact fixed-point sums, and every replica's kinetic sums
use the same 256-atom blocks as a single system)."""
import numpy as np
import pytest

from moltwister_gb300 import workloads as W
from moltwister_gb300.system import MDConfig


def shared_config(T):
    return MDConfig(timestep=0.5, ensemble="NVT", temperature=T, temperaturerelax=20.0, cutoffradius=8.5,
                    neighshell=1.0, coulomb="shifted", coulombcutoff=8.5, listskin=1.0, precision="mixed",
                    clipforces=True, optlearningrate=2e-5)


def replica_systems():
    """(systems, temperatures): two argon boxes and one water box, relaxed starts."""
    from moltwister_gb300.engine import Engine
    a1, _ = W.argon(ncell=4, seed=31, T=120.0, jitter=0.05)      # 256 atoms
    a2, _ = W.argon(ncell=5, seed=32, T=200.0, jitter=0.05)      # 500 atoms
    w, _ = W.water(n_mol=300, L=W.water_box_length(300), seed=33, T=300.0, rc=8.5)
    e = Engine(w, shared_config(300.0))
    e.optimize(200)
    w.r, _, _ = e.get_state()
    e.close()
    return [a1, w, a2], [120.0, 300.0, 200.0]


def test_shared_force_field_remaps_topology():
    from moltwister_gb300.batch import shared_force_field
    a, _ = W.argon(ncell=2, seed=1)
    w, _ = W.water(n_mol=8, L=12.0, seed=2)
    ra, rw = shared_force_field([a, w])
    assert ra.type_names() == rw.type_names() == ["Ar", "Ow", "Hw"]
    assert len(rw.bond_terms) == len(w.bond_terms) and np.array_equal(rw.bonds, w.bonds)
    assert [t.kind for t in ra.nonbonded] == [t.kind for t in rw.nonbonded]


@pytest.mark.gpu
def test_batch_replicas_match_single_runs_bitwise():
    from moltwister_gb300.batch import BatchEngine
    from moltwister_gb300.engine import Engine
    systems, temps = replica_systems()
    b = BatchEngine(systems, shared_config(300.0), temperatures=temps)
    outs = b.run_batch(200, out_stride=50)
    r, p = b.get_state()
    assert len(outs) == 4                     # steps 0, 50, 100, 150
    for k, (s, T) in enumerate(zip(systems, temps)):
        e = Engine(s, shared_config(T))
        recs = e.run(200, out_stride=50, copy_coords=False)
        rs, ps, _ = e.get_state()
        assert np.array_equal(b.replica(r, k), rs), k
        assert np.array_equal(b.replica(p, k), ps), k
        U = np.array([x.U for x in recs])
        K = np.array([x.K for x in recs])
        assert np.array_equal(np.array([o[1][k, 3] for o in outs]), U), k
        assert np.array_equal(np.array([o[1][k, 4] for o in outs]), K), k
        e.close()


@pytest.mark.gpu
def test_batch_thermostats_hold_their_temperatures():
    from moltwister_gb300.batch import BatchEngine
    systems, temps = replica_systems()
    b = BatchEngine(systems, shared_config(300.0), temperatures=temps)
    outs = b.run_batch(3000, out_stride=100)
    T_K = np.array([o[1][:, 0] for o in outs[-10:]]) * 120.272    # kJ/mol -> K, last 1,000 steps
    assert np.allclose(T_K.mean(0), temps, rtol=0.15), T_K.mean(0)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_energy_gradients_match_single_systems(prec):
    """mtg_batch_energy_grad: every replica's energy and its derivatives with respect to shared
    force-field parameters (LJ sigma and epsilon of both species, the water charge scale, bond k)
    equal those of the same replica alone (the fixed-point forces and the per-atom tangents are
    summed in a fixed order per replica; FP64 tangents)."""
    from moltwister_gb300 import grad as Gr
    from moltwister_gb300.batch import BatchEngine, shared_force_field
    from moltwister_gb300.engine import Engine
    systems, temps = replica_systems()
    cfg = shared_config(300.0)
    cfg.precision = prec
    b = BatchEngine(systems, cfg, temperatures=temps)
    ff = b.systems
    s0 = ff[1]                                  # the water replica names every type of the union
    params = [Gr.lj_sigma(s0, "Ar", "Ar"), Gr.lj_eps(s0, "Ow", "Ow"), Gr.bond_k(s0, 0)]
    U, g = b.energy_grad(params)
    for k, sk in enumerate(shared_force_field(systems)):
        ck = shared_config(temps[k])
        ck.precision = prec
        e = Engine(sk, ck)
        Uk, gk = e.energy_grad(params)
        assert abs(U[k] - Uk) <= 1e-12 * max(1.0, abs(Uk)), (k, U[k], Uk)
        assert np.allclose(g[k], gk, rtol=1e-11, atol=1e-9 * np.abs(gk).max()), (k, g[k], gk)
        e.close()
