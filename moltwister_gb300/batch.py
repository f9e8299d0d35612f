"""Batches of independent replicas advanced by the same kernel launches (mtg_batch_create).

The replicas share one force field: the union of their atom types (by name, in first-appearance
order over the replicas), of their non-bonded terms and of their bond / angle / dihedral term
types.  Each replica keeps its own box, cell grid, temperature and Nose-Hoover chain.  In mixed
precision a replica's trajectory is bit-identical to the same system run alone with `Engine`.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .engine import (Engine, MTGError, MTG_OK, OutputRecord, SystemDesc, Thermo, ThermoState, _ptr,
                     config_desc, load_library, system_desc, thermo_struct, thermo_tuple)
from .system import MDConfig, MDSystem


def _union(items, key=lambda x: x):
    out, index = [], {}
    for it in items:
        k = key(it)
        if k not in index:
            index[k] = len(out)
            out.append(it)
    return out, index


def shared_force_field(systems: Sequence[MDSystem]) -> List[MDSystem]:
    """Copies of the systems rewritten onto one shared force field (type order, non-bonded terms,
    bonded term lists with the topology's term indices remapped)."""
    names, _ = _union(n for s in systems for n in s.type_names())
    nb_all = [t for s in systems for t in s.nonbonded]
    seen = {}
    for t in nb_all:
        k = (frozenset((t.id1, t.id2)), t.kind)
        if k in seen and seen[k] != (t.args, t.cutoff):
            raise ValueError(f"replicas disagree on the {t.kind} term of {t.id1}-{t.id2}")
        seen[k] = (t.args, t.cutoff)
    nb, _ = _union(nb_all, key=lambda t: (frozenset((t.id1, t.id2)), t.kind))
    key = lambda t: (type(t).__name__, repr(t))
    bt, bidx = _union([t for s in systems for t in s.bond_terms], key)
    at, aidx = _union([t for s in systems for t in s.angle_terms], key)
    dt, didx = _union([t for s in systems for t in s.dihedral_terms], key)
    out = []
    for s in systems:
        c = s.copy()
        c.type_order = list(names)
        c.nonbonded = list(nb)
        c.bond_terms, c.angle_terms, c.dihedral_terms = list(bt), list(at), list(dt)
        if len(s.bonds):
            m = np.array([bidx[key(t)] for t in s.bond_terms], np.int32)
            c.bonds = np.asarray(s.bonds).copy()
            c.bonds[:, 2] = np.where(c.bonds[:, 2] >= 0, m[np.maximum(c.bonds[:, 2], 0)], -1)
        if len(s.angles):
            m = np.array([aidx[key(t)] for t in s.angle_terms], np.int32)
            c.angles = np.asarray(s.angles).copy()
            c.angles[:, 3] = np.where(c.angles[:, 3] >= 0, m[np.maximum(c.angles[:, 3], 0)], -1)
        if len(s.dihedrals):
            m = np.array([didx[key(t)] for t in s.dihedral_terms], np.int32)
            c.dihedrals = np.asarray(s.dihedrals).copy()
            c.dihedrals[:, 4] = np.where(c.dihedrals[:, 4] >= 0, m[np.maximum(c.dihedrals[:, 4], 0)], -1)
        out.append(c)
    return out


class BatchEngine(Engine):
    """nrep systems on one GPU, one launch per kernel per step for all of them.

    `config` is shared (precision fp64 or mixed, NVT or NVE); `temperatures` (K) and `cutoffs` (A,
    LJ and Coulomb, at most config.cutoffradius) are per replica (defaults: the config's).  Each
    replica's seeded chain state (nhT_eta / nhT_peta) is injected after creation."""

    def __init__(self, systems: Sequence[MDSystem], config: MDConfig,
                 temperatures: Optional[Sequence[float]] = None, cutoffs: Optional[Sequence[float]] = None,
                 device: int = 0):
        self.lib = load_library()
        self.config = config
        self._keep: List[object] = []
        reps = shared_force_field(systems)
        descs = [system_desc(s, self._keep) for s in reps]
        self._keep.append(descs)
        arr = (C.c_void_p * len(descs))(*[C.cast(C.pointer(d), C.c_void_p).value for d in descs])
        self._keep.append(arr)
        temps = None
        if temperatures is not None:
            temps = np.ascontiguousarray(temperatures, np.float64)
            self._keep.append(temps)
        cuts = None
        if cutoffs is not None:
            cuts = np.ascontiguousarray(cutoffs, np.float64)
            self._keep.append(cuts)
        cf = config_desc(config, device)
        self.cfgdesc = cf
        h = C.c_void_p()
        rc = self.lib.mtg_batch_create(C.cast(arr, C.c_void_p), len(descs), C.byref(cf), _ptr(temps), _ptr(cuts),
                                       C.byref(h))
        if rc != MTG_OK:
            raise MTGError(rc, self.lib.mtg_last_error(None).decode())
        self.h = h
        self.nrep = len(descs)
        self.offsets = np.zeros(self.nrep + 1, np.int32)
        self._check(self.lib.mtg_batch_info(self.h, None, _ptr(self.offsets)))
        self.n = int(self.offsets[-1])
        self.systems = reps
        if config.ensemble != "NVE":
            for r, s in enumerate(reps):
                if s.nhT_eta is not None:
                    self.set_thermo(r, Thermo(s.nhT_eta, s.nhT_peta))

    # -- per-replica state ---------------------------------------------------------------------------
    def set_thermo(self, rep: int, thermo) -> None:
        th = thermo_struct(thermo)
        self._check(self.lib.mtg_batch_set_thermo(self.h, int(rep), C.byref(th)))

    def get_thermo(self, rep: int) -> Thermo:
        th = ThermoState()
        self._check(self.lib.mtg_batch_get_thermo(self.h, int(rep), C.byref(th)))
        return thermo_tuple(th)

    def get_state(self):
        """(r, p) of all replicas, concatenated (replica r owns rows offsets[r]:offsets[r+1])."""
        r = np.zeros((self.n, 3))
        p = np.zeros((self.n, 3))
        self._check(self.lib.mtg_get_state(self.h, _ptr(r), _ptr(p), None))
        return r, p

    def set_state(self, r=None, p=None, thermo=None):
        if thermo is not None:
            raise ValueError("a batch sets chain states per replica (set_thermo)")
        Engine.set_state(self, r, p)

    def energy_grad(self, params):
        """(U [nrep], dU/dtheta [nrep, nparams]) of every replica at the current positions
        (C ABI mtg_batch_energy_grad); parameters name the shared force field (self.systems)."""
        from .engine import _param_array
        arr, keep = _param_array(params)
        U = np.zeros(self.nrep)
        g = np.zeros((self.nrep, len(params)))
        self._check(self.lib.mtg_batch_energy_grad(self.h, len(params), C.cast(arr, C.c_void_p), _ptr(U), _ptr(g)))
        return U, g

    def replica(self, a: np.ndarray, rep: int) -> np.ndarray:
        return a[self.offsets[rep]:self.offsets[rep + 1]]

    # -- dynamics ------------------------------------------------------------------------------------
    def records(self) -> np.ndarray:
        """(nrep, 6): T, P, V, U, K, E of each replica at the last output step."""
        out = np.zeros((self.nrep, 6))
        self._check(self.lib.mtg_batch_get_records(self.h, _ptr(out)))
        return out

    def run_batch(self, nsteps: int, out_stride: int = 0) -> List[Tuple[int, np.ndarray]]:
        """Runs nsteps; at every output step (step % out_stride == 0) records each replica's
        T, P, V, U, K, E.  Returns [(step, (nrep, 6) array)]."""
        outs: List[Tuple[int, np.ndarray]] = []

        def cb(rec: OutputRecord):
            outs.append((rec.step, self.records()))
            return False

        self.run(nsteps, out_stride=out_stride, callback=cb, copy_coords=False)
        return outs
