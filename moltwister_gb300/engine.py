"""ctypes binding of libmtgpu.so (C ABI: include/mtgpu.h).

`Engine(system, config)` is the Python counterpart of what `CCmdRun::execute` does with the GPU
build of MolTwister (Cmd/MolTwisterCmdMolDyn/CmdRun.cpp:121-128): describe the state once, then
run steps and receive the output scalars every `outstride` steps.  There is no CPU fallback: if
the library has not been built, importing the engine raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Callable, List, NamedTuple, Optional, Tuple

import numpy as np

from .system import (MDConfig, MDSystem, bonded_arrays, nonbonded_arrays, term_params, ENSEMBLES)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmtgpu.so")

NPTS = 1000
MAXFF = 5
MAXCHAIN = 16

PREC = {"reference": 0, "fp64": 1, "mixed": 2}
COULOMB = {"allpairs": 0, "cutoff": 1, "shifted": 2}

MTG_OK = 0
MTG_E_INVALID = -1
ERRORS = {-1: "invalid", -2: "cuda", -3: "nomem", -4: "overflow", -5: "timeout", -6: "unsupported", -7: "nonfinite"}


class MTGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mtgpu error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("p", C.c_double * 4)]


class SystemDesc(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("n_types", C.c_int32),
                ("r", C.c_void_p), ("p", C.c_void_p), ("mass", C.c_void_p), ("charge", C.c_void_p),
                ("type", C.c_void_p), ("mol", C.c_void_p), ("mobile", C.c_void_p),
                ("box", C.c_double * 3),
                ("nb_count", C.c_void_p), ("nb_terms", C.c_void_p), ("nb_tables", C.c_void_p),
                ("n_bond_types", C.c_int32), ("bond_terms", C.c_void_p), ("bond_tables", C.c_void_p),
                ("n_angle_types", C.c_int32), ("angle_terms", C.c_void_p), ("angle_tables", C.c_void_p),
                ("n_dih_types", C.c_int32), ("dih_terms", C.c_void_p), ("dih_tables", C.c_void_p),
                ("n_bonds", C.c_int32), ("bonds", C.c_void_p),
                ("n_angles", C.c_int32), ("angles", C.c_void_p),
                ("n_dihedrals", C.c_int32), ("dihedrals", C.c_void_p)]


class ConfigDesc(C.Structure):
    _fields_ = [("ensemble", C.c_int32), ("temperature_nh_len", C.c_int32), ("temperature_respa", C.c_int32),
                ("pressure_nh_len", C.c_int32), ("pressure_respa", C.c_int32), ("precision", C.c_int32),
                ("coulomb", C.c_int32), ("clip_forces", C.c_int32),
                ("timestep", C.c_double), ("temperature", C.c_double), ("temperature_relax", C.c_double),
                ("pressure", C.c_double), ("pressure_relax", C.c_double), ("cutoff_radius", C.c_double),
                ("neigh_shell", C.c_double), ("cutoff_force", C.c_double),
                ("scale12", C.c_double), ("scale13", C.c_double), ("scale14", C.c_double), ("scale1N", C.c_double),
                ("coulomb_cutoff", C.c_double), ("list_skin", C.c_double),
                ("opt_learning_rate", C.c_double), ("opt_accuracy", C.c_double), ("opt_max_steps", C.c_int32),
                ("device", C.c_int32), ("lj_shift", C.c_int32), ("initial_max_neighbours", C.c_int32)]


class ThermoState(C.Structure):
    _fields_ = [("M", C.c_int32), ("reserved", C.c_int32), ("eta", C.c_double * MAXCHAIN),
                ("p_eta", C.c_double * MAXCHAIN), ("p_eps", C.c_double), ("eps", C.c_double),
                ("MP", C.c_int32), ("reserved2", C.c_int32), ("etaP", C.c_double * MAXCHAIN),
                ("p_etaP", C.c_double * MAXCHAIN), ("box", C.c_double * 3)]


class Thermo(NamedTuple):
    """Thermostat chain (eta, peta) and, under NPT, the barostat: p_eps, strain eps, its chain
    (etaP, petaP) and the current box (output only)."""
    eta: np.ndarray
    peta: np.ndarray
    p_eps: float = 0.0
    eps: float = 0.0
    etaP: Optional[np.ndarray] = None
    petaP: Optional[np.ndarray] = None
    box: Optional[np.ndarray] = None


class Param(C.Structure):
    _fields_ = [("kind", C.c_int32), ("index", C.c_int32), ("dq", C.c_void_p)]


class LossDesc(C.Structure):
    _fields_ = [("nsteps", C.c_int32), ("checkpoint_every", C.c_int32), ("type_a", C.c_int32),
                ("type_b", C.c_int32), ("nbins", C.c_int32), ("reserved", C.c_int32),
                ("rmax", C.c_double), ("width", C.c_double), ("target", C.c_void_p)]


class Output(C.Structure):
    _fields_ = [("step", C.c_int64), ("T", C.c_double), ("P", C.c_double), ("V", C.c_double),
                ("U", C.c_double), ("K", C.c_double), ("E", C.c_double),
                ("r", C.c_void_p), ("p", C.c_void_p)]


class RunStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("steps", C.c_int64), ("list_builds", C.c_int64),
                ("kernel_launches", C.c_int64), ("graph_steps", C.c_int32), ("force_team", C.c_int32),
                ("graph_form", C.c_int32)]


OUTPUT_CB = C.CFUNCTYPE(C.c_int, C.POINTER(Output), C.c_void_p)

_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libmtgpu.so and declares the C signatures.  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m moltwister_gb300.build` "
                           "(there is no CPU fallback)")
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "mtg_version": ([], C.c_int),
        "mtg_device_name": ([C.c_int, C.c_char_p, C.c_int], C.c_int),
        "mtg_term_profile": ([C.POINTER(Term), C.c_float, C.c_float, C.c_int, P], C.c_int),
        "mtg_create": ([C.POINTER(SystemDesc), C.POINTER(ConfigDesc), C.POINTER(P)], C.c_int),
        "mtg_destroy": ([P], None),
        "mtg_last_error": ([P], C.c_char_p),
        "mtg_set_state": ([P, P, P, C.POINTER(ThermoState)], C.c_int),
        "mtg_get_state": ([P, P, P, C.POINTER(ThermoState)], C.c_int),
        "mtg_run": ([P, C.c_int, C.c_int, OUTPUT_CB, P], C.c_int),
        "mtg_optimize": ([P, C.c_double, C.c_int, C.c_int, OUTPUT_CB, P], C.c_int),
        "mtg_compute_forces": ([P, P, P, P], C.c_int),
        "mtg_get_cells": ([P, P, P, P, P, C.c_int32, P], C.c_int),
        "mtg_get_neighbors": ([P, C.c_int32, P, P, P], C.c_int),
        "mtg_get_run_stats": ([P, C.POINTER(RunStats)], C.c_int),
        "mtg_profile_phases": ([P, C.c_int, P], C.c_int),
        "mtg_set_wait_limit": ([P, C.c_int32], C.c_int),
        "mtg_draw_initial_state": ([C.POINTER(SystemDesc), C.POINTER(ConfigDesc), C.c_uint32, C.c_int32, P,
                                    C.POINTER(ThermoState)], C.c_int),
        "mtg_init_state": ([P, C.c_uint32, C.c_int32], C.c_int),
        "mtg_neighbors_noalloc": ([P, C.c_int32, P, C.c_double, C.c_double, C.c_int32, P, P, P, P], C.c_int),
        "mtg_batch_create": ([P, C.c_int32, C.POINTER(ConfigDesc), P, P, C.POINTER(P)], C.c_int),
        "mtg_batch_info": ([P, P, P], C.c_int),
        "mtg_batch_get_records": ([P, P], C.c_int),
        "mtg_batch_set_thermo": ([P, C.c_int32, C.POINTER(ThermoState)], C.c_int),
        "mtg_batch_get_thermo": ([P, C.c_int32, C.POINTER(ThermoState)], C.c_int),
        "mtg_get_params": ([P, C.c_int32, P, P], C.c_int),
        "mtg_set_params": ([P, C.c_int32, P, P], C.c_int),
        "mtg_energy_grad": ([P, C.c_int32, P, P, P], C.c_int),
        "mtg_batch_energy_grad": ([P, C.c_int32, P, P, P], C.c_int),
        "mtg_loss_grad": ([P, C.POINTER(LossDesc), C.c_int32, P, P, P, P], C.c_int),
        "mtg_pair_histogram": ([P, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, P], C.c_int),
        "mtg_dcd_append": ([C.c_char_p, C.c_int32, P, P, C.c_int32, C.c_int32, C.c_double], C.c_int),
        "mtg_xyz_append": ([C.c_char_p, C.c_int32, P, P, C.c_int32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def term_profile(term, x0: float, x1: float, npts: int = NPTS) -> np.ndarray:
    """Host-side table of one MDFF term record (C ABI mtg_term_profile)."""
    lib = load_library()
    kind, p = term_params(term)
    t = Term(kind, 0, (C.c_double * 4)(*p))
    out = np.zeros((npts, 3), np.float32)
    rc = lib.mtg_term_profile(C.byref(t), float(np.float32(x0)), float(np.float32(x1)), npts, _ptr(out))
    if rc != MTG_OK:
        raise MTGError(rc, "mtg_term_profile failed")
    return out


@dataclass
class OutputRecord:
    step: int
    T: float
    P: float
    V: float
    U: float
    K: float
    E: float
    r: Optional[np.ndarray] = None
    p: Optional[np.ndarray] = None


def _terms_array(terms) -> C.Array:
    arr = (Term * max(len(terms), 1))()
    for i, t in enumerate(terms):
        k, p = term_params(t)
        arr[i].kind = k
        for w in range(4):
            arr[i].p[w] = p[w]
    return arr


def thermo_struct(thermo) -> ThermoState:
    if not isinstance(thermo, Thermo):
        thermo = Thermo(*thermo)
    th = ThermoState()
    th.M = len(thermo.eta)
    for j in range(len(thermo.eta)):
        th.eta[j] = float(thermo.eta[j])
        th.p_eta[j] = float(thermo.peta[j])
    th.p_eps, th.eps = float(thermo.p_eps), float(thermo.eps)
    if thermo.etaP is not None:
        th.MP = len(thermo.etaP)
        for j in range(th.MP):
            th.etaP[j] = float(thermo.etaP[j])
            th.p_etaP[j] = float(thermo.petaP[j])
    if thermo.box is not None:
        for a in range(3):
            th.box[a] = float(thermo.box[a])
    return th


def thermo_tuple(th: ThermoState) -> Thermo:
    return Thermo(np.array(th.eta[:th.M]), np.array(th.p_eta[:th.M]), th.p_eps, th.eps,
                  np.array(th.etaP[:th.MP]), np.array(th.p_etaP[:th.MP]), np.array(th.box[:]))


def system_desc(s: MDSystem, keep_list: List[object], tables: Optional[dict] = None) -> SystemDesc:
    """mtg_system_desc of an MDSystem; the arrays it points to are appended to keep_list."""
    n = s.n

    def keep(a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        keep_list.append(a)
        return a

    counts, kinds, params = nonbonded_arrays(s)
    T = counts.shape[0]
    nb_terms = (Term * (T * T * MAXFF))()
    _, pair_terms = s.nonbonded_pair_terms()
    for pr in range(T * T):
        for ff, t in enumerate(pair_terms[pr]):
            k, p = term_params(t)
            nb_terms[pr * MAXFF + ff].kind = k
            for w in range(4):
                nb_terms[pr * MAXFF + ff].p[w] = p[w]
    keep_list.append(nb_terms)
    bt, at, dt = _terms_array(s.bond_terms), _terms_array(s.angle_terms), _terms_array(s.dihedral_terms)
    keep_list.extend([bt, at, dt])
    d = SystemDesc()
    d.n_atoms, d.n_types = n, T
    d.r = _ptr(keep(s.r, np.float64))
    d.p = _ptr(keep(s.p, np.float64)) if s.p is not None else None
    d.mass = _ptr(keep(s.m, np.float64))
    d.charge = _ptr(keep(s.q, np.float64))
    d.type = _ptr(keep(s.type_index(), np.int32))
    d.mol = _ptr(keep(s.mol_index(), np.int32))
    d.mobile = _ptr(keep(s.mobile, np.uint8))
    for a in range(3):
        d.box[a] = float(s.box[a])
    d.nb_count = _ptr(keep(counts.reshape(-1), np.int32))
    d.nb_terms = C.cast(nb_terms, C.c_void_p).value
    d.n_bond_types, d.bond_terms = len(s.bond_terms), C.cast(bt, C.c_void_p).value
    d.n_angle_types, d.angle_terms = len(s.angle_terms), C.cast(at, C.c_void_p).value
    d.n_dih_types, d.dih_terms = len(s.dihedral_terms), C.cast(dt, C.c_void_p).value
    if tables is not None:
        d.nb_tables = _ptr(keep(tables["nb"], np.float32))
        d.bond_tables = _ptr(keep(tables["bond"], np.float32)) if len(s.bond_terms) else None
        d.angle_tables = _ptr(keep(tables["angle"], np.float32)) if len(s.angle_terms) else None
        d.dih_tables = _ptr(keep(tables["dih"], np.float32)) if len(s.dihedral_terms) else None
    d.n_bonds, d.bonds = len(s.bonds), _ptr(keep(np.asarray(s.bonds).reshape(-1, 3), np.int32))
    d.n_angles, d.angles = len(s.angles), _ptr(keep(np.asarray(s.angles).reshape(-1, 4), np.int32))
    d.n_dihedrals, d.dihedrals = len(s.dihedrals), _ptr(keep(np.asarray(s.dihedrals).reshape(-1, 5), np.int32))
    return d


def config_desc(c: MDConfig, device: int = 0) -> ConfigDesc:
    """mtg_config_desc of an MDConfig (the moldyn cfg keys plus the new ones)."""
    cf = ConfigDesc()
    cf.ensemble = ENSEMBLES[c.ensemble]
    cf.temperature_nh_len, cf.temperature_respa = c.temperaturenhlen, c.temperaturerespa
    cf.pressure_nh_len, cf.pressure_respa = c.pressurenhlen, c.pressurerespa
    cf.precision = PREC[c.precision]
    cf.coulomb = COULOMB[c.coulomb]
    cf.clip_forces = 1 if c.clipforces else 0
    cf.timestep, cf.temperature, cf.temperature_relax = c.timestep, c.temperature, c.temperaturerelax
    cf.pressure, cf.pressure_relax = c.pressure, c.pressurerelax
    cf.cutoff_radius, cf.neigh_shell, cf.cutoff_force = c.cutoffradius, c.neighshell, c.cutoffforce
    cf.scale12, cf.scale13, cf.scale14, cf.scale1N = c.scale12, c.scale13, c.scale14, c.scale1N
    cf.coulomb_cutoff = c.coulombcutoff if c.coulombcutoff is not None else c.cutoffradius
    cf.list_skin = c.listskin
    cf.opt_learning_rate, cf.opt_accuracy, cf.opt_max_steps = c.optlearningrate, c.optaccuracy, c.optmaxsteps
    cf.device = device
    cf.lj_shift = int(c.ljshift)
    cf.initial_max_neighbours = int(getattr(c, "initialmaxneighbours", 0))
    return cf



class Engine:
    """One MD system on one GPU.

    tables: optional dict with "nb" ((T*T*5, 1000, 3) float32, this project's pair-major layout),
    "bond", "angle", "dih" ((ntypes, 1000, 3)); when absent the library tabulates the terms itself.
    """

    def __init__(self, system: MDSystem, config: MDConfig, tables: Optional[dict] = None, device: int = 0):
        self.lib = load_library()
        self.system, self.config = system, config
        s, c = system, config
        self._keep: List[object] = []
        d = system_desc(s, self._keep, tables)
        self.desc = d
        cf = config_desc(c, device)
        self.cfgdesc = cf
        h = C.c_void_p()
        rc = self.lib.mtg_create(C.byref(d), C.byref(cf), C.byref(h))
        if rc != MTG_OK:
            raise MTGError(rc, self.lib.mtg_last_error(None).decode())
        self.h = h
        self.n = s.n
        if c.ensemble == "NPT" and s.p_eps is not None:
            M = c.temperaturenhlen
            self.set_state(thermo=Thermo(s.nhT_eta if s.nhT_eta is not None else np.zeros(M),
                                         s.nhT_peta if s.nhT_peta is not None else np.zeros(M),
                                         float(s.p_eps), 0.0, s.nhP_eta, s.nhP_peta))
        elif s.nhT_eta is not None and c.ensemble != "NVE":
            self.set_state(thermo=(s.nhT_eta, s.nhT_peta))

    # -- lifetime ----------------------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.mtg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != MTG_OK:
            raise MTGError(rc, self.lib.mtg_last_error(self.h).decode())

    # -- state ---------------------------------------------------------------------------------------
    def set_state(self, r=None, p=None, thermo=None):
        rr = None if r is None else np.ascontiguousarray(r, np.float64)
        pp = None if p is None else np.ascontiguousarray(p, np.float64)
        th = None
        if thermo is not None:
            th = thermo_struct(thermo)
        self._check(self.lib.mtg_set_state(self.h, _ptr(rr), _ptr(pp), C.byref(th) if th is not None else None))

    def get_state(self, out=None):
        """(r, p, Thermo) after the last completed step.  `out` = (r, p): C-contiguous float64
        [n, 3] arrays to fill (for instance views of pinned host memory) instead of new ones."""
        if out is not None:
            r, p = out
            for a in (r, p):
                if a.dtype != np.float64 or a.shape != (self.n, 3) or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError("get_state(out=...) needs C-contiguous float64 arrays of shape (n, 3)")
        else:
            r = np.zeros((self.n, 3))
            p = np.zeros((self.n, 3))
        th = ThermoState()
        self._check(self.lib.mtg_get_state(self.h, _ptr(r), _ptr(p), C.byref(th)))
        return r, p, thermo_tuple(th)


    # -- dynamics ------------------------------------------------------------------------------------
    def run(self, nsteps: int, out_stride: int = 0, callback: Optional[Callable[[OutputRecord], bool]] = None,
            copy_coords: bool = True) -> List[OutputRecord]:
        """Runs nsteps; returns the output records (every out_stride steps, step % stride == 0)."""
        records: List[OutputRecord] = []
        n = self.n

        def _cb(op, user):
            o = op.contents
            rec = OutputRecord(int(o.step), o.T, o.P, o.V, o.U, o.K, o.E)
            if copy_coords:
                rec.r = np.ctypeslib.as_array(C.cast(o.r, C.POINTER(C.c_double)), shape=(n, 3)).copy()
                rec.p = np.ctypeslib.as_array(C.cast(o.p, C.POINTER(C.c_double)), shape=(n, 3)).copy()
            records.append(rec)
            if callback is not None:
                return 1 if callback(rec) else 0
            return 0

        cb = OUTPUT_CB(_cb) if out_stride > 0 else OUTPUT_CB()
        self._check(self.lib.mtg_run(self.h, int(nsteps), int(out_stride), cb, None))
        return records

    def optimize(self, max_steps: int, accuracy: float = 0.0, out_stride: int = 0,
                 callback: Optional[Callable[[OutputRecord], bool]] = None) -> List[OutputRecord]:
        """Gradient-descent minimisation with the config's learning rate (C ABI mtg_optimize)."""
        records: List[OutputRecord] = []

        def _cb(op, user):
            o = op.contents
            rec = OutputRecord(int(o.step), o.T, o.P, o.V, o.U, o.K, o.E)
            records.append(rec)
            return 1 if (callback is not None and callback(rec)) else 0

        cb = OUTPUT_CB(_cb) if out_stride > 0 else OUTPUT_CB()
        self._check(self.lib.mtg_optimize(self.h, float(accuracy), int(max_steps), int(out_stride), cb, None))
        return records

    # -- parameters and gradients ---------------------------------------------------------------
    def get_params(self, params) -> np.ndarray:
        arr, keep = _param_array(params)
        out = np.zeros(len(params))
        self._check(self.lib.mtg_get_params(self.h, len(params), C.cast(arr, C.c_void_p), _ptr(out)))
        return out

    def set_params(self, params, values) -> None:
        arr, keep = _param_array(params)
        v = np.ascontiguousarray(values, np.float64)
        self._check(self.lib.mtg_set_params(self.h, len(params), C.cast(arr, C.c_void_p), _ptr(v)))

    def energy_grad(self, params) -> Tuple[float, np.ndarray]:
        """(U, dU/dtheta) at the current positions."""
        arr, keep = _param_array(params)
        U = np.zeros(1)
        g = np.zeros(len(params))
        self._check(self.lib.mtg_energy_grad(self.h, len(params), C.cast(arr, C.c_void_p), _ptr(U), _ptr(g)))
        return float(U[0]), g

    def loss_grad(self, loss, params, with_grad: bool = True) -> Tuple[float, np.ndarray, np.ndarray]:
        """(L, dL/dtheta, gbar) of a pair-correlation trajectory loss (mtg_loss_grad); `loss` has
        the fields of mtg_loss_desc (see moltwister_gb300.grad.RDFLoss).  with_grad=False evaluates
        the loss only."""
        arr, keep = _param_array(params)
        tgt = np.ascontiguousarray(loss.target, np.float64)
        d = LossDesc(int(loss.nsteps), int(loss.checkpoint_every), int(loss.type_a), int(loss.type_b),
                     int(loss.nbins), 0, float(loss.rmax), float(loss.width), tgt.ctypes.data)
        L = np.zeros(1)
        g = np.zeros(len(params))
        gbar = np.zeros(int(loss.nbins))
        self._check(self.lib.mtg_loss_grad(self.h, C.byref(d), len(params), C.cast(arr, C.c_void_p), _ptr(L),
                                           _ptr(g) if with_grad else None, _ptr(gbar)))
        return float(L[0]), g, gbar

    def pair_histogram(self, type_a: int, type_b: int, nbins: int, rmin: float, rmax: float,
                       ignore_below: float = -1.0, profile: Optional[np.ndarray] = None) -> np.ndarray:
        """Adds the current frame's ordered-pair distance counts to profile (int64[nbins])."""
        prof = np.zeros(nbins, np.int64) if profile is None else profile
        self._check(self.lib.mtg_pair_histogram(self.h, int(type_a), int(type_b), int(nbins), float(rmin), float(rmax),
                                                float(ignore_below), _ptr(prof)))
        return prof

    def stats(self) -> dict:
        st = RunStats()
        self._check(self.lib.mtg_get_run_stats(self.h, C.byref(st)))
        return {"device_ms": st.device_ms, "steps": st.steps, "list_builds": st.list_builds,
                "kernel_launches": st.kernel_launches, "graph_steps": st.graph_steps,
                "force_team": st.force_team, "graph_form": st.graph_form}

    def init_state(self, seed: int = 1, mode: str = "reference") -> None:
        """Draw and set the initial momenta and chain state (C ABI mtg_init_state); see
        draw_initial_state for the modes."""
        self._check(self.lib.mtg_init_state(self.h, int(seed) & 0xFFFFFFFF, INIT_MODES[mode]))

    def set_wait_limit(self, polls: int) -> None:
        """Poll limit of the bounded device waits (C ABI mtg_set_wait_limit); 0 = give up at once."""
        self._check(self.lib.mtg_set_wait_limit(self.h, int(polls)))

    def profile_phases(self, steps: int) -> dict:
        """Mean device ms per step of each phase (C ABI mtg_profile_phases)."""
        out = np.zeros(5)
        self._check(self.lib.mtg_profile_phases(self.h, int(steps), _ptr(out)))
        return {"kick_drift": out[0], "list": out[1], "force": out[2], "kick_reduce": out[3], "step_end": out[4]}

    # -- parity hooks ----------------------------------------------------------------------------------
    def forces(self):
        F = np.zeros((self.n, 3))
        U = np.zeros(self.n)
        self._check(self.lib.mtg_compute_forces(self.h, _ptr(F), None, _ptr(U)))
        return F, U

    def cells(self):
        dims = np.zeros(3, np.int32)
        self._check(self.lib.mtg_get_cells(self.h, _ptr(dims), None, None, None, 0, None))
        nc = int(np.prod(dims))
        ixyz = np.zeros((self.n, 3), np.int32)
        first = np.zeros(nc, np.int32)
        count = np.zeros(nc, np.int32)
        lst = np.zeros(self.n, np.int32)
        self._check(self.lib.mtg_get_cells(self.h, _ptr(dims), _ptr(ixyz), _ptr(first), _ptr(count), nc, _ptr(lst)))
        return dims, ixyz, first, count, lst

    def neighbors(self):
        count = np.zeros(self.n, np.int32)
        need = np.zeros(1, np.int32)
        self._check(self.lib.mtg_get_neighbors(self.h, 0, _ptr(count), None, _ptr(need)))
        m = max(int(need[0]), 1)
        lst = np.zeros((self.n, m), np.int32)
        self._check(self.lib.mtg_get_neighbors(self.h, m, _ptr(count), _ptr(lst), _ptr(need)))
        return count, lst


def _param_array(params):
    """ctypes mtg_param array of (kind, index, dq) tuples; returns (array, arrays kept alive)."""
    arr = (Param * max(len(params), 1))()
    keep = []
    for k, (kind, index, dq) in enumerate(params):
        arr[k].kind, arr[k].index = int(kind), int(index)
        if dq is not None:
            a = np.ascontiguousarray(dq, np.float64)
            keep.append(a)
            arr[k].dq = a.ctypes.data
    keep.append(arr)
    return arr, keep


INIT_MODES = {"reference": 0, "maxwell": 1}


def draw_initial_state(system: MDSystem, config: MDConfig, seed: int = 1, mode: str = "reference"):
    """(p [n, 3], Thermo) as mtg_draw_initial_state draws them on the host: "reference" is the
    state MolTwister's CSimulationBox constructor draws after srand(seed); "maxwell" a seeded
    Maxwell-Boltzmann state."""
    lib = load_library()
    keep: List[object] = []
    sd = system_desc(system, keep)
    cd = config_desc(config)
    p = np.zeros((system.n, 3))
    th = ThermoState()
    rc = lib.mtg_draw_initial_state(C.byref(sd), C.byref(cd), int(seed) & 0xFFFFFFFF, INIT_MODES[mode], _ptr(p),
                                    C.byref(th))
    if rc != MTG_OK:
        raise MTGError(rc, lib.mtg_last_error(None).decode())
    return p, thermo_tuple(th)


def neighbors_noalloc(r_ptr: int, n: int, box, cutoff: float, shell: float, max_neigh: int,
                      count_ptr: int, list_ptr: int, stream: int = 0, wait: bool = True):
    """Reference-order neighbour list of device-resident positions through
    mtg_neighbors_noalloc (no context, no device allocation).  Pointers are device addresses of
    the current device (e.g. a CUDA tensor's data_ptr()); `stream` a cudaStream_t handle.
    Returns the largest count when some list was truncated to max_neigh, 0 when all fit, or
    None when wait is False (the call then only enqueues work)."""
    lib = load_library()
    b = (C.c_double * 3)(*[float(x) for x in box])
    need = C.c_int32(0)
    rc = lib.mtg_neighbors_noalloc(C.c_void_p(r_ptr), int(n), b, float(cutoff), float(shell), int(max_neigh),
                                   C.c_void_p(count_ptr), C.c_void_p(list_ptr) if list_ptr else None,
                                   C.byref(need) if wait else None, C.c_void_p(stream) if stream else None)
    if rc != MTG_OK:
        raise MTGError(rc, lib.mtg_last_error(None).decode())
    return int(need.value) if wait else None


def device_name(device: int = 0) -> str:
    lib = load_library()
    buf = C.create_string_buffer(256)
    if lib.mtg_device_name(device, buf, 256) != MTG_OK:
        return "unknown"
    return buf.value.decode()
