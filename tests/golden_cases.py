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


def neighbour_hash(count: np.ndarray, lists: np.ndarray) -> np.ndarray:
    """One 64-bit FNV-1a hash per atom over its ordered neighbour indices (int32, little endian
    bytes), for fixtures too large to store whole lists: equal hashes and counts stand for equal
    ordered lists.  `lists` is [n, >= max(count)]; entries past an atom's count are ignored."""
    count = np.asarray(count, np.int64)
    lists = np.asarray(lists)
    h = np.full(count.shape[0], 0xCBF29CE484222325, np.uint64)
    prime = np.uint64(0x100000001B3)
    width = int(count.max()) if count.size else 0
    with np.errstate(over="ignore"):
        for col in range(width):
            live = col < count
            v = lists[:, col].astype(np.int64).astype(np.uint32)
            g = h.copy()
            for b in range(4):
                g = (g ^ ((v >> np.uint32(8 * b)) & np.uint32(0xFF)).astype(np.uint64)) * prime
            h = np.where(live, g, h)
    return h


def neighbours_match(d, cnt: np.ndarray, lst: np.ndarray) -> bool:
    """Ordered neighbour lists equal to a fixture's (whole lists, or hashes for the large cases)."""
    if not np.array_equal(cnt, d["neigh_count"]):
        return False
    if "neigh_hash" in d:
        return bool(np.array_equal(neighbour_hash(cnt, lst), d["neigh_hash"]))
    for k in range(cnt.shape[0]):
        if not np.array_equal(lst[k, :cnt[k]], d["neigh_list"][k, :cnt[k]]):
            return False
    return True


def names():
    # every fixture but the initial-state and pair-correlation ones is a system with its reference run
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("init_", "paircorr_")))


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
