"""TEST INFRASTRUCTURE: ctypes wrapper around the C oracle (oracle/mdoracle.c).

Only tests/, __graft_entry__.smoke() and bench.py (CPU-baseline and reference legs) use this module,
and only as the checker or the timed CPU baseline.  The product library never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

from moltwister_gb300.system import (MDConfig, MDSystem, bonded_arrays, cell_counts,
                                     nonbonded_arrays, per_atom_lists)

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmdoracle.so")
NPTS = 1000
MAXFF = 5
CONV_T = 120.272
CONV_PRESS = 16388.2461


def build(force: bool = False) -> str:
    """Compile libmdoracle.so (gcc -O2 -ffp-contract=off: no fused multiply-adds, as the reference's
    x86-64 build; OpenMP over atoms, whose sums do not depend on the thread count)."""
    src = os.path.join(HERE, "mdoracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src, "-lm"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        P = C.c_void_p
        for name in ("orc_profile_nb", "orc_profile_bond", "orc_profile_angle", "orc_profile_dih"):
            f = getattr(_lib, name)
            f.argtypes = [C.c_int, P, C.c_float, C.c_float, C.c_int, P]
            f.restype = C.c_int
        _lib.orc_cell_list.argtypes = [C.c_int, P, P, C.c_int, C.c_int, C.c_int, P, P, P]
        _lib.orc_neigh_list.argtypes = [C.c_int, P, P, C.c_float, C.c_int, C.c_int, C.c_int, P, P, P, C.c_int, P, P]
        _lib.orc_neigh_list.restype = C.c_int
        _lib.orc_forces_ref.argtypes = [P, P, P, C.c_int, P, P]
        _lib.orc_forces_fp64.argtypes = [P, C.c_double, P, P]
        _lib.orc_forces_fp64_vir.argtypes = [P, C.c_double, P, P, P]
        _lib.orc_run_ref.argtypes = [P, P, P, P, P, P, P, C.c_int, C.c_int, P, P, P, P]
        _lib.orc_run_ref.restype = C.c_int
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class OrcSys(C.Structure):
    _fields_ = [("n", C.c_int), ("ntypes", C.c_int),
                ("r", C.c_void_p), ("q", C.c_void_p), ("m", C.c_void_p), ("type", C.c_void_p),
                ("mol", C.c_void_p), ("mobile", C.c_void_p),
                ("box", C.c_double * 3),
                ("rc", C.c_float), ("shell", C.c_float), ("fcut", C.c_float),
                ("scale12", C.c_float), ("scale13", C.c_float), ("scale14", C.c_float), ("scale1N", C.c_float),
                ("nb_tab", C.c_void_p), ("nb_cnt", C.c_void_p),
                ("bond_tab", C.c_void_p), ("angle_tab", C.c_void_p), ("dih_tab", C.c_void_p),
                ("bptr", C.c_void_p), ("bj", C.c_void_p), ("bt", C.c_void_p),
                ("aptr", C.c_void_p), ("ai", C.c_void_p), ("aj", C.c_void_p), ("at", C.c_void_p), ("acen", C.c_void_p),
                ("dptr", C.c_void_p), ("di", C.c_void_p), ("dj", C.c_void_p), ("dl", C.c_void_p), ("dt", C.c_void_p),
                ("dcen", C.c_void_p),
                ("nb_kind", C.c_void_p), ("nb_par", C.c_void_p),
                ("bond_kind", C.c_void_p), ("bond_par", C.c_void_p),
                ("angle_kind", C.c_void_p), ("angle_par", C.c_void_p),
                ("dih_kind", C.c_void_p), ("dih_par", C.c_void_p),
                ("coulomb_mode", C.c_int), ("coulomb_rc", C.c_double), ("qd", C.c_void_p), ("lj_shift", C.c_int)]


class OrcRun(C.Structure):
    _fields_ = [("ensemble", C.c_int), ("dt", C.c_double), ("kT", C.c_double), ("tau", C.c_double),
                ("M", C.c_int), ("nresp", C.c_int), ("fcut", C.c_double),
                ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("MP", C.c_int), ("nrespP", C.c_int), ("tauP", C.c_double), ("Pext", C.c_double)]


def profile(kind_group: str, kind: int, params, x0: float, x1: float, npts: int = NPTS) -> np.ndarray:
    out = np.zeros((npts, 3), np.float32)
    p = np.asarray(list(params) + [0.0] * (4 - len(params)), np.float64)
    getattr(lib(), "orc_profile_" + kind_group)(kind, _p(p), x0, x1, npts, _p(out))
    return out


def tables(s: MDSystem, cfg: MDConfig):
    """Oracle tables: nb (T*T*5, 1000, 3), bond/angle/dih (ntype, 1000, 3), in the layout
    [((row*T + col)*5 + ff)] of this project (the reference stores the point index outermost)."""
    counts, kinds, params = nonbonded_arrays(s)
    T = counts.shape[0]
    rc = np.float32(cfg.cutoffradius)
    nb = np.zeros((T * T * MAXFF, NPTS, 3), np.float32)
    for pr in range(T * T):
        for ff in range(int(counts.reshape(-1)[pr])):
            nb[pr * MAXFF + ff] = profile("nb", int(kinds.reshape(-1, MAXFF)[pr, ff]),
                                          params.reshape(-1, MAXFF, 4)[pr, ff], np.float32(0.01), rc)
    two_pi = np.float32(2.0 * np.pi)
    bk, bp = bonded_arrays(s.bond_terms)
    ak, ap = bonded_arrays(s.angle_terms)
    dk, dp = bonded_arrays(s.dihedral_terms)
    bond = np.stack([profile("bond", int(k), p, np.float32(0.01), rc) for k, p in zip(bk, bp)]) if len(bk) else np.zeros((0, NPTS, 3), np.float32)
    ang = np.stack([profile("angle", int(k), p, np.float32(0.0), two_pi) for k, p in zip(ak, ap)]) if len(ak) else np.zeros((0, NPTS, 3), np.float32)
    dih = np.stack([profile("dih", int(k), p, np.float32(0.0), two_pi) for k, p in zip(dk, dp)]) if len(dk) else np.zeros((0, NPTS, 3), np.float32)
    return {"nb": nb, "nb_count": counts.astype(np.int32), "bond": bond, "angle": ang, "dih": dih}


def reference_nb_layout(nb_table_ref: np.ndarray, T: int) -> np.ndarray:
    """Convert the reference's point-outermost non-bonded table (index T*(T*(5*j+ff)+row)+col,
    MDFFMatrices.cpp:538-541) to this project's [((row*T+col)*5+ff), j] layout."""
    a = nb_table_ref.reshape(NPTS, MAXFF, T, T, 3)          # [j, ff, row, col, 3]
    return np.ascontiguousarray(a.transpose(2, 3, 1, 0, 4)).reshape(T * T * MAXFF, NPTS, 3)


class Oracle:
    """Holds the flattened arrays of one system and exposes the oracle functions."""

    def __init__(self, s: MDSystem, cfg: MDConfig, tabs: Optional[dict] = None,
                 bonds=None, angles=None, dihedrals=None, mol=None):
        self.s, self.cfg = s, cfg
        n = s.n
        self.r = np.ascontiguousarray(s.r, np.float64).copy()
        self.q = np.ascontiguousarray(s.q, np.float32)          # reference keeps q as float
        self.qd = np.ascontiguousarray(s.q, np.float64)
        self.m = np.ascontiguousarray(s.m, np.float64)
        self.type = s.type_index().astype(np.int32)
        self.mol = np.ascontiguousarray(s.mol_index() if mol is None else mol, np.int32)
        self.mobile = np.ascontiguousarray(s.mobile, np.int32)
        self.tabs = tabs if tabs is not None else tables(s, cfg)
        counts, kinds, params = nonbonded_arrays(s)
        self.nb_kind = np.ascontiguousarray(kinds.reshape(-1), np.int32)
        self.nb_par = np.ascontiguousarray(params.reshape(-1, 4), np.float64)
        self.nb_cnt = np.ascontiguousarray(self.tabs["nb_count"].reshape(-1), np.int32)
        self.bond_kind, self.bond_par = bonded_arrays(s.bond_terms)
        self.angle_kind, self.angle_par = bonded_arrays(s.angle_terms)
        self.dih_kind, self.dih_par = bonded_arrays(s.dihedral_terms)
        bonds = s.bonds if bonds is None else bonds
        angles = s.angles if angles is None else angles
        dihedrals = s.dihedrals if dihedrals is None else dihedrals
        self.lists = per_atom_lists(n, bonds, angles, dihedrals)
        self.nb_tab = np.ascontiguousarray(self.tabs["nb"], np.float32)
        self.bond_tab = np.ascontiguousarray(self.tabs["bond"], np.float32)
        self.angle_tab = np.ascontiguousarray(self.tabs["angle"], np.float32)
        self.dih_tab = np.ascontiguousarray(self.tabs["dih"], np.float32)
        self.cells = cell_counts(s.box, cfg.cutoffradius, cfg.neighshell)
        self._keep = []
        self.st = self._make_struct()

    def _make_struct(self) -> OrcSys:
        s, cfg, L = self.s, self.cfg, self.lists
        o = OrcSys()
        o.n, o.ntypes = self.s.n, len(self.s.type_names())
        arrays = dict(r=self.r, q=self.q, qd=self.qd, m=self.m, type=self.type, mol=self.mol, mobile=self.mobile,
                      nb_tab=self.nb_tab, nb_cnt=self.nb_cnt, bond_tab=self.bond_tab,
                      angle_tab=self.angle_tab, dih_tab=self.dih_tab,
                      nb_kind=self.nb_kind, nb_par=self.nb_par,
                      bond_kind=self.bond_kind.astype(np.int32), bond_par=self.bond_par,
                      angle_kind=self.angle_kind.astype(np.int32), angle_par=self.angle_par,
                      dih_kind=self.dih_kind.astype(np.int32), dih_par=self.dih_par)
        arrays.update({k: np.ascontiguousarray(v, np.int32) for k, v in L.items()})
        for k, v in arrays.items():
            v = np.ascontiguousarray(v)
            if v.size == 0:
                v = np.zeros(1, v.dtype)
            self._keep.append(v)
            setattr(o, k, v.ctypes.data)
        for a in range(3):
            o.box[a] = float(s.box[a])
        o.rc, o.shell, o.fcut = cfg.cutoffradius, cfg.neighshell, cfg.cutoffforce
        o.scale12, o.scale13, o.scale14, o.scale1N = cfg.scale12, cfg.scale13, cfg.scale14, cfg.scale1N
        o.coulomb_mode = {"allpairs": 0, "cutoff": 1, "shifted": 2}[cfg.coulomb]
        o.lj_shift = int(getattr(cfg, "ljshift", 0))
        o.coulomb_rc = cfg.coulombcutoff if cfg.coulombcutoff is not None else cfg.cutoffradius
        return o

    def set_positions(self, r: np.ndarray):
        self.r[...] = r
        return self

    # -- lists -------------------------------------------------------------------------------
    def cell_list(self, r: Optional[np.ndarray] = None):
        r = self.r if r is None else np.ascontiguousarray(r, np.float64)
        n = self.s.n
        nx, ny, nz = self.cells
        Lf = np.asarray(self.s.box, np.float32)
        ac = np.zeros((n, 3), np.int32)
        cp = np.zeros((nx * ny * nz, 2), np.int32)
        cl = np.zeros(n, np.int32)
        lib().orc_cell_list(n, _p(r), _p(Lf), nx, ny, nz, _p(ac), _p(cp), _p(cl))
        return ac, cp, cl

    def neigh_list(self, r: Optional[np.ndarray] = None):
        r = self.r if r is None else np.ascontiguousarray(r, np.float64)
        n = self.s.n
        ac, cp, cl = self.cell_list(r)
        nx, ny, nz = self.cells
        Lf = np.asarray(self.s.box, np.float32)
        cnt = np.zeros(n, np.int32)
        need = lib().orc_neigh_list(n, _p(r), _p(Lf), self.cfg.cutoffradius, nx, ny, nz,
                                    _p(ac), _p(cp), _p(cl), 0, _p(cnt), None)
        maxn = max(need, 1)
        lst = np.full((n, maxn), -1, np.int32)
        lib().orc_neigh_list(n, _p(r), _p(Lf), self.cfg.cutoffradius, nx, ny, nz,
                             _p(ac), _p(cp), _p(cl), maxn, _p(cnt), _p(lst))
        return cnt, lst

    # -- forces ------------------------------------------------------------------------------
    def forces_ref(self):
        cnt, lst = self.neigh_list()
        n = self.s.n
        F = np.zeros((n, 3), np.float64)
        U = np.zeros(n, np.float32)
        lib().orc_forces_ref(C.byref(self.st), _p(cnt), _p(lst), lst.shape[1], _p(F), _p(U))
        return F, U

    def forces_fp64(self, rcut: Optional[float] = None):
        n = self.s.n
        F = np.zeros((n, 3), np.float64)
        U = np.zeros(n, np.float64)
        lib().orc_forces_fp64(C.byref(self.st), float(self.cfg.cutoffradius if rcut is None else rcut), _p(F), _p(U))
        return F, U

    # -- dynamics ----------------------------------------------------------------------------
    def run_ref(self, nsteps: int, stride: int, p: Optional[np.ndarray] = None):
        s, cfg = self.s, self.cfg
        n = s.n
        r = self.r
        p = np.ascontiguousarray((s.p if p is None else p), np.float64).copy()
        M = cfg.temperaturenhlen
        eta = np.ascontiguousarray(s.nhT_eta if s.nhT_eta is not None else np.zeros(M), np.float64).copy()
        peta = np.ascontiguousarray(s.nhT_peta if s.nhT_peta is not None else np.zeros(M), np.float64).copy()
        MP = cfg.pressurenhlen
        baro = np.zeros(2 + 2 * MP)
        baro[0] = s.p_eps if s.p_eps is not None else 0.0
        if s.nhP_eta is not None:
            baro[2:2 + MP] = s.nhP_eta
        if s.nhP_peta is not None:
            baro[2 + MP:] = s.nhP_peta
        rc = OrcRun()
        rc.ensemble = {"NVT": 0, "NPT": 1, "NVE": 2}[cfg.ensemble]
        rc.MP, rc.nrespP = MP, cfg.pressurerespa
        rc.tauP = cfg.pressurerelax / 100.0
        rc.Pext = cfg.pressure / CONV_PRESS
        rc.dt = cfg.timestep / 100.0
        rc.kT = cfg.temperature / CONV_T
        rc.tau = cfg.temperaturerelax / 100.0
        rc.M, rc.nresp = M, cfg.temperaturerespa
        rc.fcut = cfg.cutoffforce
        rc.nx, rc.ny, rc.nz = self.cells
        nrec = 2 + nsteps // stride
        rr = np.zeros((nrec, n, 3)); rp = np.zeros((nrec, n, 3)); rF = np.zeros((nrec, n, 3)); rs = np.zeros((nrec, 5))
        got = lib().orc_run_ref(C.byref(self.st), C.byref(rc), _p(r), _p(p), _p(eta), _p(peta), _p(baro),
                                nsteps, stride, _p(rr), _p(rp), _p(rF), _p(rs))
        if got < 0:
            raise RuntimeError("oracle run failed")
        return {"r": rr[:got], "p": rp[:got], "F": rF[:got], "scal": rs[:got], "eta": eta, "peta": peta,
                "p_eps": baro[0], "eps": baro[1], "etaP": baro[2:2 + MP], "petaP": baro[2 + MP:]}
