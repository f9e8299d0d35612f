"""Generates the golden fixtures in this folder from the reference's own CPU MD code.

Run from the repository root after building the oracle harness (needs the reference sources):

    make -C oracle/ref REF=<MolTwister source tree> && python tests/golden/make_golden.py [case ...]

Each case is a seeded synthetic system (moltwister_gb300/workloads.py).  The harness
(oracle/ref/harness.cpp, linked from the unmodified reference sources) builds the
CMolTwisterState through the reference API and records:
  static : the 1000-point tables, the bonded lists the reference discovers, the cell list, the
           full neighbour list and per-atom F/U at the input positions;
  run    : a trajectory of `steps` steps (r, p, F every `stride` steps plus U, K, T, P, V and the
           Nose-Hoover chain), with momenta and chain variables injected from the seeded system.
The inputs are stored next to the outputs so the GPU tests can rebuild the system on a machine
without the reference.
"""
from __future__ import annotations

import dataclasses
import json
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from moltwister_gb300 import workloads as W  # noqa: E402
from oracle.sysfile import harness_run, harness_static  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def cases():
    """name -> (system, config, steps, stride)"""
    out = {}
    s, c = W.argon(ncell=5, seed=11, jitter=0.05)
    c.neighshell = 1.0                      # 3 cells per axis
    out["argon500_nvt"] = (s, c, 100, 25)
    s, c = W.argon(ncell=5, seed=12, jitter=0.05, T=90.0)
    c.neighshell = 1.0
    c.ensemble = "NVE"
    out["argon500_nve"] = (s, c, 100, 25)
    s, c = W.argon(ncell=4, seed=13, jitter=0.05)
    out["argon256_2cells"] = (s, c, 20, 10)   # 2 cells per axis: duplicated neighbours (reference trap)
    s, c = W.water(n_mol=216, L=W.water_box_length(216), seed=14, rc=6.0)
    c.neighshell = 0.2
    out["water648_nvt"] = (s, c, 100, 25)
    s, c = W.chains(n_chain=27, L=24.0, seed=15, immobile_every=7)
    out["chains108_nvt"] = (s, c, 100, 25)
    # NPT (VelVerlet.cpp:57-71).  The reference's barostat is driven by sum F.r over wrapped
    # positions (VelVerlet.cpp:160-174), not the pair virial, so the default 5 ps relaxation time
    # collapses or explodes these boxes within ~100 steps; slow barostats keep 100 steps finite.
    s, c = W.argon(ncell=5, seed=11, jitter=0.05)
    c.neighshell = 1.0
    c.pressurerelax = 100000.0
    W.make_npt(s, c, 500.0, 21)
    out["argon500_npt"] = (s, c, 100, 25)
    s, c = W.water(n_mol=216, L=W.water_box_length(216), seed=14, rc=6.0)
    c.neighshell = 0.2
    c.pressurerelax = 20000.0
    W.make_npt(s, c, 1.0, 22)
    out["water648_npt"] = (s, c, 100, 25)
    return out


def big_cases():
    """The two full-size parity cases (4,000-atom argon, 9,000-atom water).  Their neighbour lists are stored as one 64-bit hash
    per atom (golden_cases.neighbour_hash) and their trajectories without forces, which keeps the
    fixtures near a megabyte each."""
    out = {}
    # argon, 4,000 atoms: FCC 10^3 cells, cutoff 2.5 sigma, shell 2 A -> 5^3 cells, NVT, dt 2 fs
    s, c = W.argon(ncell=10, seed=1)
    out["argon4000_nvt"] = (s, c, 100, 50)
    # flexible water, 9,000 atoms in a 44.8 A box, reference all-pairs Coulomb, 10 A cutoff and
    # shell 2 A -> 3^3 cells, NVT 300 K, dt 0.5 fs.  The lattice start releases enough energy to
    # drive the reference's chain to NaN within 50 steps, so the start is first relaxed by the
    # reference's own gradient descent (`moldyn optimizeenergy`, SimulationBox.cpp:197-208)
    s, c = W.water(n_mol=3000, L=44.8, seed=2, rc=10.0, dt=0.5)
    s.r = relax_reference(s, c, steps=300, lr=2e-5)
    out["water9000_ref"] = (s, c, 100, 50)
    return out


def relax_reference(s, c, steps, lr):
    """r <- r + lr F for `steps` steps with the reference-precision forces (the oracle, which the
    fixtures pin bit for bit to the reference build), then wrapped into the box."""
    from oracle import oracle as O
    orc = O.Oracle(s, c)
    r = np.array(s.r, dtype=np.float64)
    for _ in range(steps):
        orc.set_positions(r)
        F, _ = orc.forces_ref()
        r = r + lr * F
    return r - s.box * np.floor(r / s.box + 0.5)


def pack(name, s, c, steps, stride, big=False):
    st = harness_static(s, c)
    tr = harness_run(s, c, steps, stride)
    cnt = st["neigh_count"]
    maxc = int(cnt.max()) if cnt.size else 0
    if big:
        from tests.golden_cases import neighbour_hash
        nb = dict(neigh_count=cnt, neigh_hash=neighbour_hash(cnt, st["neigh_list"][:, :maxc]),
                  neigh_max=np.array(maxc))
        traj = dict(traj_r=tr["traj_r"], traj_p=tr["traj_p"])
        # a short prefix (one record) that the CPU oracle can replay within seconds
        k = 10 if s.n <= 4000 else 4
        pre = harness_run(s, c, k, k)
        traj.update(prefix_steps=np.array(k), prefix_r=pre["traj_r"][-1], prefix_p=pre["traj_p"][-1],
                    prefix_scalars=pre["traj_scalars"][-1])
    else:
        nb = dict(neigh_count=cnt, neigh_list=st["neigh_list"][:, :maxc])
        traj = dict(traj_r=tr["traj_r"], traj_p=tr["traj_p"], traj_F=tr["traj_F"], traj_U=tr["traj_U"])
    terms = {
        "nonbonded": [dataclasses.asdict(t) for t in s.nonbonded],
        "bond_terms": [dataclasses.asdict(t) for t in s.bond_terms],
        "angle_terms": [dataclasses.asdict(t) for t in s.angle_terms],
        "dihedral_terms": [dataclasses.asdict(t) for t in s.dihedral_terms],
    }
    cfg = dataclasses.asdict(c)
    arrays = dict(
        in_box=s.box, in_ids=np.array(s.ids), in_r=s.r, in_q=s.q, in_m=s.m, in_mobile=s.mobile.astype(np.int8),
        in_p=s.p, in_nhT_eta=s.nhT_eta, in_nhT_peta=s.nhT_peta,
        in_p_eps=np.array(np.nan if s.p_eps is None else s.p_eps),
        in_nhP_eta=np.zeros(0) if s.nhP_eta is None else s.nhP_eta,
        in_nhP_peta=np.zeros(0) if s.nhP_peta is None else s.nhP_peta,
        in_terms=np.array(json.dumps(terms)), in_cfg=np.array(json.dumps(cfg)),
        steps=np.array(steps), stride=np.array(stride),
        nb_table=st["nb_table"], nb_count=st["nb_count"], bond_table=st["bond_table"],
        angle_table=st["angle_table"], dih_table=st["dih_table"],
        atom_type=st["atom_type"], atom_mol=st["atom_mol"],
        bonds=st["bonds"], angles=st["angles"], dihedrals=st["dihedrals"],
        cell_dims=st["cell_dims"], atom_cell=st["atom_cell"], cell_ptr=st["cell_ptr"], cell_list=st["cell_list"],
        F=st["F"], U=st["U"], **nb, **traj,
        traj_scalars=tr["traj_scalars"], traj_nhT=tr["traj_nhT"],
        traj_nhP=tr["traj_nhP"], traj_peps=tr["traj_peps"],
    )
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrays)
    return path


def make_dcd(name="water648_nvt"):
    """dcd_<name>.bin: two records written by the reference's CDCDFile (the system's positions and
    the same shifted by +0.125 A), header for 100 steps every 25 at dt 0.5 fs."""
    import tempfile
    from oracle.sysfile import run_harness
    s, c, _, _ = cases()[name]
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.dcd")
        run_harness(["dcd", out, 100, 25, 0.5], s, c)
        data = open(out, "rb").read()
    path = os.path.join(OUT, f"dcd_{name}.bin")
    with open(path, "wb") as fh:
        fh.write(data)
    return path


def init_cases():
    """(name, system, config, seed) of the initial-state fixture: mixed masses with immobile atoms,
    one mass, and an NPT configuration (barostat chain and momentum)."""
    out = []
    s, c = W.chains(n_chain=27, L=24.0, seed=15, immobile_every=7)
    out += [("chains108_seed1", s, c, 1), ("chains108_seed12345", s, c, 12345)]
    s, c = W.argon(ncell=5, seed=11, jitter=0.05)
    out.append(("argon500_seed1", s, c, 1))
    s, c = W.water(n_mol=216, L=W.water_box_length(216), seed=14, rc=6.0)
    c.ensemble = "NPT"
    out.append(("water648_npt_seed7", s, c, 7))
    return out


def make_init():
    """init_states.npz: per case the reference's drawn momenta, chains and barostat momentum, with
    the inputs that determine them (masses, mobility, configuration)."""
    from oracle.sysfile import harness_init
    arrays = {}
    for name, s, c, seed in init_cases():
        d = harness_init(s, c, seed)
        arrays[f"{name}__m"] = s.m
        arrays[f"{name}__mobile"] = s.mobile.astype(np.int8)
        arrays[f"{name}__cfg"] = np.array(json.dumps(dataclasses.asdict(c)))
        arrays[f"{name}__seed"] = np.array(seed)
        for k in ("init_p", "init_nhT", "init_nhP", "init_peps"):
            arrays[f"{name}__{k}"] = d[k]
    path = os.path.join(OUT, "init_states.npz")
    np.savez_compressed(path, **arrays)
    return path


PAIRCORR_CASES = [("Ow_Hw", ["Ow", "Hw", "120", "0.0", "9.0"]),
                  ("Ow_Ow_ignore", ["Ow", "Ow", "90", "0.0", "9.0", "ignoredistbelow", "2.5"]),
                  ("Hw_Hw_nopbc", ["Hw", "Hw", "60", "0.5", "12.0", "ignorepbc"])]


def make_paircorr(name="water648_nvt", nframes=3, shift=0.37):
    """paircorr_<name>.npz: the reference's `calculate paircorrelation` table (counts and its
    PairCorr / RDF columns) over a DCD of nframes frames, frame f = the case's positions + f shift,
    for the argument lists of PAIRCORR_CASES, with the PBC widths the command read."""
    import tempfile
    from oracle.analysis import read_pair_correlation
    from oracle.sysfile import run_harness
    from tests.golden_cases import load
    s, c, _ = load(name)
    arrays = {"nframes": np.array(nframes), "shift": np.array(shift)}
    with tempfile.TemporaryDirectory() as td:
        for key, args in PAIRCORR_CASES:
            out = os.path.join(td, key + ".txt")
            run_harness(["paircorr", out, nframes, shift] + args, s, c)
            table, pbc = read_pair_correlation(out)
            arrays[key + "__args"] = np.array(json.dumps(args))
            arrays[key + "__table"] = table
            arrays[key + "__pbc"] = pbc
    path = os.path.join(OUT, f"paircorr_{name}.npz")
    np.savez_compressed(path, **arrays)
    return path


def main(only=()):
    todo = [(k, v, False) for k, v in cases().items()] + [(k, v, True) for k, v in big_cases().items()]
    for name, (s, c, steps, stride), big in todo:
        if only and name not in only:
            continue
        p = pack(name, s, c, steps, stride, big=big)
        print(f"{name}: {os.path.getsize(p) / 1024:.0f} KiB")


if __name__ == "__main__":
    if sys.argv[1:] == ["dcd"]:
        print(make_dcd())
    elif sys.argv[1:] == ["init"]:
        print(make_init())
    elif sys.argv[1:] == ["paircorr"]:
        print(make_paircorr())
    else:
        main(tuple(sys.argv[1:]))
