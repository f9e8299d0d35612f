"""Loads the golden fixtures of tests/golden/ (written by tests/golden/make_golden.py from the
reference's own CPU MD code) back into MDSystem / MDConfig objects plus the reference outputs."""
from __future__ import annotations

import glob
import json
import os
from typing import Dict, Tuple

import numpy as np

from moltwister_gb300.system import (AngleTerm, BondTerm, DihedralTerm, MDConfig, MDSystem,
                                     NonBondedTerm)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name: str) -> Tuple[MDSystem, MDConfig, Dict[str, np.ndarray]]:
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    terms = json.loads(str(d["in_terms"]))
    cfgd = json.loads(str(d["in_cfg"]))
    cfg = MDConfig(**cfgd)
    tup = lambda t: {**t, "args": tuple(t["args"])}
    s = MDSystem(box=d["in_box"], ids=[str(x) for x in d["in_ids"]], r=d["in_r"], q=d["in_q"], m=d["in_m"],
                 mobile=d["in_mobile"].astype(bool),
                 nonbonded=[NonBondedTerm(**tup(t)) for t in terms["nonbonded"]],
                 bond_terms=[BondTerm(**tup(t)) for t in terms["bond_terms"]],
                 angle_terms=[AngleTerm(**tup(t)) for t in terms["angle_terms"]],
                 dihedral_terms=[DihedralTerm(**tup(t)) for t in terms["dihedral_terms"]])
    # the topology the reference discovered (its order fixes the per-atom list order)
    s.bonds = d["bonds"].reshape(-1, 3).astype(np.int32)
    s.angles = d["angles"].reshape(-1, 4).astype(np.int32)
    s.dihedrals = d["dihedrals"].reshape(-1, 5).astype(np.int32)
    s.mol = d["atom_mol"].astype(np.int32)
    s.p = d["in_p"]
    s.nhT_eta = d["in_nhT_eta"]
    s.nhT_peta = d["in_nhT_peta"]
    if "in_p_eps" in d and np.isfinite(d["in_p_eps"]):
        s.p_eps = float(d["in_p_eps"])
        s.nhP_eta = d["in_nhP_eta"]
        s.nhP_peta = d["in_nhP_peta"]
    return s, cfg, d
