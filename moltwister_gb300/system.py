"""Host-side description of an MD system, mirroring what MolTwister's `moldyn run` consumes.

The reference keeps its inputs in `CMolTwisterState` (atoms with ID, position, charge `Q_`, mass `m_`,
`isMobile_`; MolTwisterState.h:84-94, MolTwisterAtom.h:144-149) and in the four MDFF lists filled by the
`add mdnonbonded|mdbond|mdangle|mddihedral` commands (Cmd/MolTwisterCmdAdd/CmdMDNonBonded.cpp:72-114,
CmdMDBond.cpp:81-152, CmdMDAngle.cpp, CmdMDDihedral.cpp).  Run settings live in `SMolDynConfigStruct`
(Cmd/MolTwisterCmdMolDyn/Config/MolDynConfigStruct.h:24-65) set through `moldyn cfg set <key> <value>`
(Config/MolDynConfig.cpp:95-287, defaults :289-328).

`MDSystem` holds the same information as plain numpy arrays plus MDFF term records that keep the
reference's command-line argument order, so a system can be written out for the reference harness
(`oracle/sysfile.py`) and passed to the GPU library through the C ABI (`moltwister_gb300.engine`).

Atom types are numbered in first-appearance order of the atom IDs, as
`CMolTwisterState::searchForAtomTypes` does (MolTwisterState.cpp:459-487).
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# Term kinds; the integer values are the MTG_* kind codes of include/mtgpu.h.
NB_KINDS = {"LJ": 1, "LJ1208": 2, "Buck": 3, "LJBuck": 4}
BOND_KINDS = {"Harm": 11, "Morse": 12, "LJC": 13}
ANGLE_KINDS = {"Harm": 21, "Class2": 22}
DIH_KINDS = {"Harm": 31, "Fourier4t": 32}


@dataclass
class NonBondedTerm:
    """One `add mdnonbonded ID1 ID2 TYPE args...` entry (CmdMDNonBonded.cpp:72-114).

    Argument order per type, as the reference parses it:
      LJ   : epsilon sigma [alpha a]       (MolTwisterMDFFNonBonded_LJ.cpp:44-58; alpha defaults to 1)
      Buck : A rho C                        (MolTwisterMDFFNonBonded_Buck.cpp)
    """
    id1: str
    id2: str
    kind: str
    args: Tuple[float, ...]
    cutoff: float = 0.0   # new, production modes only: this pair's cutoff [A] (0 = cutoffradius)

    def params(self) -> List[float]:
        if self.kind == "LJ":
            eps, sig = self.args[0], self.args[1]
            alpha = self.args[2] if len(self.args) > 2 else 1.0
            return [eps, sig, alpha, float(self.cutoff)]
        return list(self.args)

    def command_args(self) -> List[str]:
        if self.kind == "LJ" and len(self.args) > 2:
            return [repr(float(self.args[0])), repr(float(self.args[1])), "alpha", repr(float(self.args[2]))]
        return [repr(float(a)) for a in self.args]


@dataclass
class BondTerm:
    """One `add mdbond ID1 ID2 TYPE [criterion R0] args...` entry (CmdMDBond.cpp:81-152).

    Harm: k r0 with U = k (r - r0)^2 (MolTwisterMDFFBond_Harm.cpp:90-97, no factor 1/2).
    Morse: D alpha r0.
    """
    id1: str
    id2: str
    kind: str
    args: Tuple[float, ...]
    criterion: str = "all_r_less_than"
    crit_r0: float = 1.75


@dataclass
class AngleTerm:
    """One `add mdangle ID1 ID2 ID3 TYPE [criterion R0] args...` entry.

    Harm: k theta0[deg] with U = k (theta - theta0)^2 (MolTwisterMDFFAngle_Harm.cpp:94-108).
    """
    id1: str
    id2: str
    id3: str
    kind: str
    args: Tuple[float, ...]
    criterion: str = "all_r_less_than"
    crit_r0: float = 1.75


@dataclass
class DihedralTerm:
    """One `add mddihedral ID1 ID2 ID3 ID4 TYPE [criterion R0] args...` entry.

    Harm: K D N with U = K (1 + D cos(N phi)); Fourier4t: V1 V2 V3 V4.
    """
    id1: str
    id2: str
    id3: str
    id4: str
    kind: str
    args: Tuple[float, ...]
    criterion: str = "all_r_less_than"
    crit_r0: float = 1.75


# SMolDynConfigStruct defaults (Config/MolDynConfig.cpp:289-328).  Keys follow `moldyn cfg set`.
ENSEMBLES = {"NVT": 0, "NPT": 1, "NVE": 2}


@dataclass
class MDConfig:
    """Mirror of `SMolDynConfigStruct` with the reference defaults, plus the new engine's own keys.

    Reference keys (names as in `moldyn cfg set`): timestep [fs], timesteps, outstride, ensemble,
    temperature [K], temperaturerelax [fs], temperaturenhlen, temperaturerespa, pressure [atm],
    pressurerelax [fs], pressurenhlen, pressurerespa, cutoffradius [A], neighshell [A], cutoffforce,
    scale12, scale13, scale14, scale1N, optmaxsteps, optlearningrate, optaccuracy.

    New keys (no counterpart in the reference):
      precision     : "reference" (tables, reference arithmetic; the parity mode),
                      "fp64" (analytic FP64), "mixed" (FP32 arithmetic, int64 fixed-point forces).
      coulomb       : "allpairs" (the reference: minimum image, no cutoff), "cutoff" (truncated at
                      coulombcutoff) or "shifted" (shifted force, smooth at coulombcutoff).
      coulombcutoff : cutoff radius for "cutoff" Coulomb [A] (defaults to cutoffradius).
      listskin      : Verlet skin of the production neighbour list [A].
      clipforces    : apply the reference's per-component force clipping (NVT/NVE only).
      ljshift       : production modes, LJ at each term's cutoff: 0 truncated (the reference),
                      1 energy shifted to zero (forces unchanged), 2 force shifted (force and
                      energy continuous: smooth trajectories for gradients).
      initialmaxneighbours : first capacity of the neighbour lists per atom (the reference starts
                      at 10, MDFFMatrices.cpp:246); 0 sizes them from the density.  Lists that
                      overflow grow and the step is redone.
    """
    timestep: float = 1.0
    timesteps: int = 50000
    outstride: int = 100
    ensemble: str = "NVT"
    temperature: float = 298.0
    temperaturerelax: float = 20.0
    temperaturenhlen: int = 4
    temperaturerespa: int = 4
    pressure: float = 1.0
    pressurerelax: float = 5000.0
    pressurenhlen: int = 4
    pressurerespa: int = 4
    cutoffradius: float = 10.0
    neighshell: float = 2.0
    cutoffforce: float = 1000.0
    scale12: float = 0.0
    scale13: float = 0.0
    scale14: float = 0.5
    scale1N: float = 0.0
    optmaxsteps: int = 5000
    optlearningrate: float = 1e-6
    optaccuracy: float = 0.0
    # new keys
    precision: str = "reference"
    coulomb: str = "allpairs"
    coulombcutoff: Optional[float] = None
    listskin: float = 1.0
    clipforces: bool = True
    ljshift: int = 0
    initialmaxneighbours: int = 0

    REFERENCE_KEYS = ("timestep", "timesteps", "outstride", "temperature", "temperaturerelax",
                      "temperaturenhlen", "temperaturerespa", "pressure", "pressurerelax",
                      "pressurenhlen", "pressurerespa", "cutoffradius", "neighshell", "cutoffforce",
                      "scale12", "scale13", "scale14", "scale1N", "optmaxsteps", "optlearningrate",
                      "optaccuracy")

    def reference_cfg_lines(self) -> List[Tuple[str, str]]:
        """(key, value) pairs for `moldyn cfg set`, in an order where `timestep` precedes the keys
        whose defaults the reference derives from it."""
        out = [("ensemble", self.ensemble.lower())]
        for k in self.REFERENCE_KEYS:
            v = getattr(self, k)
            out.append((k, repr(float(v)) if isinstance(v, float) else str(v)))
        return out


@dataclass
class MDSystem:
    box: np.ndarray                       # (3,) periodic box widths [A]; box spans [-L/2, L/2)
    ids: List[str]                        # atom IDs (names)
    r: np.ndarray                         # (N,3) float64 positions [A]
    q: np.ndarray                         # (N,) charges [e]
    m: np.ndarray                         # (N,) masses [g/mol]
    mobile: np.ndarray                    # (N,) bool
    nonbonded: List[NonBondedTerm] = field(default_factory=list)
    bond_terms: List[BondTerm] = field(default_factory=list)
    angle_terms: List[AngleTerm] = field(default_factory=list)
    dihedral_terms: List[DihedralTerm] = field(default_factory=list)
    # Explicit topology (what CMolTwisterStateTools::getAllMD*InSystem discovers in the reference):
    bonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))      # (i, j, term)
    angles: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))     # (i, center, k, term)
    dihedrals: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.int32))  # (i, j, k, l, term)
    mol: Optional[np.ndarray] = None      # (N,) molecule index, -1 for none
    p: Optional[np.ndarray] = None        # (N,3) momenta [g/mol * A / (100 fs)]
    nhT_eta: Optional[np.ndarray] = None
    nhT_peta: Optional[np.ndarray] = None
    # NPT: barostat momentum p_eps (CVelVerlet::p_eps_) and the barostat's chain (NH_P_)
    p_eps: Optional[float] = None
    nhP_eta: Optional[np.ndarray] = None
    nhP_peta: Optional[np.ndarray] = None
    # Atom-type numbering; None = first appearance of the IDs (MolTwisterState.cpp:459-487).  A batch
    # of replicas sets one shared order so that all replicas index the same force field.
    type_order: Optional[List[str]] = None

    @property
    def n(self) -> int:
        return int(self.r.shape[0])

    def type_names(self) -> List[str]:
        if self.type_order is not None:
            return list(self.type_order)
        seen: Dict[str, int] = {}
        for a in self.ids:
            if a not in seen:
                seen[a] = len(seen)
        return list(seen.keys())

    def type_index(self) -> np.ndarray:
        names = {t: i for i, t in enumerate(self.type_names())}
        return np.array([names[a] for a in self.ids], dtype=np.int32)

    def mol_index(self) -> np.ndarray:
        if self.mol is not None:
            return np.asarray(self.mol, dtype=np.int32)
        return np.full(self.n, -1, dtype=np.int32)

    def copy(self) -> "MDSystem":
        return dataclasses.replace(
            self, box=self.box.copy(), ids=list(self.ids), r=self.r.copy(), q=self.q.copy(),
            m=self.m.copy(), mobile=self.mobile.copy(),
            bonds=self.bonds.copy(), angles=self.angles.copy(), dihedrals=self.dihedrals.copy(),
            mol=None if self.mol is None else self.mol.copy(),
            p=None if self.p is None else self.p.copy(),
            nhT_eta=None if self.nhT_eta is None else self.nhT_eta.copy(),
            nhT_peta=None if self.nhT_peta is None else self.nhT_peta.copy(),
            nhP_eta=None if self.nhP_eta is None else self.nhP_eta.copy(),
            nhP_peta=None if self.nhP_peta is None else self.nhP_peta.copy())

    def nonbonded_pair_terms(self, max_per_pair: int = 5) -> Tuple[np.ndarray, List[List[NonBondedTerm]]]:
        """Per (row, col) type pair, the MDFF non-bonded entries that apply, in list order.

        Mirrors CMDFFNonBondedList::indexFromNames (MolTwisterMDFFNonBondedList.cpp:85-111), which
        matches the pair in either order, and the `add` rule that an entry with the same atom pair
        and type replaces the earlier one (MolTwisterMDFFList.h:50-76).
        """
        # Apply add/replace semantics to get the effective list.
        eff: List[NonBondedTerm] = []
        for t in self.nonbonded:
            hit = -1
            for i, e in enumerate(eff):
                same_pair = (e.id1 == t.id1 and e.id2 == t.id2) or (e.id1 == t.id2 and e.id2 == t.id1)
                if same_pair and e.kind == t.kind:
                    hit = i
                    break
            if hit >= 0:
                eff[hit] = t
            else:
                eff.append(t)
        names = self.type_names()
        T = len(names)
        counts = np.zeros((T, T), dtype=np.int32)
        terms: List[List[NonBondedTerm]] = [[] for _ in range(T * T)]
        for r_ in range(T):
            for c in range(T):
                lst = [e for e in eff if (e.id1 == names[c] and e.id2 == names[r_]) or
                       (e.id1 == names[r_] and e.id2 == names[c])]
                if len(lst) > max_per_pair:
                    raise ValueError(f"more than {max_per_pair} non-bonded terms for pair "
                                     f"({names[r_]}, {names[c]})")
                counts[r_, c] = len(lst)
                terms[r_ * T + c] = lst
        return counts, terms


TO_RAD = 0.017453292519943295   # CMDFFAngle_Harm::toRad_ (MolTwisterMDFFAngle_Harm.h:36)


def term_params(term) -> Tuple[int, List[float]]:
    """(kind code, 4 parameters) of an MDFF term record, in the order the kernels read them.

    Non-bonded LJ/LJ1208: (eps, sigma, alpha); Buck: (A, rho, C).  Bond Harm: (k, r0);
    Morse: (D, alpha, r0).  Angle Harm: (k, theta0 [deg], toRad).  Dihedral Harm: (K, D, N);
    Fourier4t: (V1, V2, V3, V4).  Kinds without an analytic form (LJBuck, LJC, Class2) are still
    accepted: their forces come from the 1000-point tables in every precision mode.
    """
    if isinstance(term, NonBondedTerm):
        kind = NB_KINDS[term.kind]
        p = term.params()
    elif isinstance(term, BondTerm):
        kind = BOND_KINDS[term.kind]
        p = list(term.args)
    elif isinstance(term, AngleTerm):
        kind = ANGLE_KINDS[term.kind]
        p = list(term.args)
        if term.kind == "Harm":
            p = [term.args[0], term.args[1], TO_RAD]
    elif isinstance(term, DihedralTerm):
        kind = DIH_KINDS[term.kind]
        p = list(term.args)
    else:
        raise TypeError(term)
    p = [float(x) for x in p][:4]
    return kind, p + [0.0] * (4 - len(p))


def nonbonded_arrays(sys_: "MDSystem"):
    """counts (T,T) int32, kinds (T,T,5) int32, params (T,T,5,4) float64 for the type-pair terms."""
    counts, terms = sys_.nonbonded_pair_terms()
    T = counts.shape[0]
    kinds = np.zeros((T, T, 5), np.int32)
    params = np.zeros((T, T, 5, 4), np.float64)
    for pr in range(T * T):
        for ff, t in enumerate(terms[pr]):
            k, p = term_params(t)
            kinds[pr // T, pr % T, ff] = k
            params[pr // T, pr % T, ff] = p
    return counts, kinds, params


def bonded_arrays(terms):
    """kinds (n,) int32 and params (n,4) float64 for a list of bond/angle/dihedral term records."""
    kinds = np.zeros(max(len(terms), 0), np.int32)
    params = np.zeros((len(terms), 4), np.float64)
    for i, t in enumerate(terms):
        kinds[i], params[i] = term_params(t)
    return kinds, params


def cell_counts(box, rc: float, shell: float) -> Tuple[int, int, int]:
    """Cells per axis, as CMDFFMatrices::CCellList::init computes them (MDFFMatrices.cpp:45-58):
    floor(double(float(L) / (float(rc) + float(shell))))."""
    R = np.float32(rc) + np.float32(shell)
    return tuple(int(math.floor(float(np.float32(L) / R))) for L in box)


def per_atom_lists(n: int, bonds: np.ndarray, angles: np.ndarray, dihedrals: np.ndarray):
    """Per-atom bonded lists in the reference's order (MDFFMatrices.cpp:384-520).

    Returns CSR arrays: bonds (ptr, partner, type); angles (ptr, i, j, type, centre);
    dihedrals (ptr, i, j, l, type, centre).  Entries for atom k follow the order of the global
    lists; for an angle (a1, a2, a3) atom k=a1 gets (a2, a3), k=a2 (the centre) gets (a1, a3),
    k=a3 gets (a2, a1); for a dihedral (a1..a4) k=a1 gets (a2, a3, a4), k=a2 gets (a1, a3, a4),
    k=a3 gets (a4, a2, a1), k=a4 gets (a3, a2, a1); centres are a2 and a3.
    """
    def csr(rows):
        rows.sort(key=lambda t: (t[0], t[1]))     # stable by (atom, global order)
        ptr = np.zeros(n + 1, np.int32)
        for t in rows:
            ptr[t[0] + 1] += 1
        return np.cumsum(ptr).astype(np.int32), rows

    b_rows = []
    for j, (a, b, t) in enumerate(np.asarray(bonds).reshape(-1, 3)):
        if t < 0:
            continue
        b_rows.append((int(a), j, int(b), int(t)))
        if b != a:
            b_rows.append((int(b), j, int(a), int(t)))
    bptr, b_rows = csr(b_rows)
    a_rows = []
    for j, (a1, a2, a3, t) in enumerate(np.asarray(angles).reshape(-1, 4)):
        if t < 0:
            continue
        for k in {int(a1), int(a2), int(a3)}:
            I = J = -1
            cen = 0
            if a1 == k:
                I, J = a2, a3
            if a2 == k:
                cen, I, J = 1, a1, a3
            if a3 == k:
                I, J = a2, a1
            a_rows.append((k, j, int(I), int(J), int(t), cen))
    aptr, a_rows = csr(a_rows)
    d_rows = []
    for j, (a1, a2, a3, a4, t) in enumerate(np.asarray(dihedrals).reshape(-1, 5)):
        if t < 0:
            continue
        for k in {int(a1), int(a2), int(a3), int(a4)}:
            I = J = L = -1
            cen = 0
            if a1 == k:
                I, J, L = a2, a3, a4
            if a2 == k:
                cen, I, J, L = 1, a1, a3, a4
            if a3 == k:
                cen, I, J, L = 1, a4, a2, a1
            if a4 == k:
                I, J, L = a3, a2, a1
            d_rows.append((k, j, int(I), int(J), int(L), int(t), cen))
    dptr, d_rows = csr(d_rows)
    col = lambda rows, c: np.array([r[c] for r in rows], np.int32)
    return {
        "bptr": bptr, "bj": col(b_rows, 2), "bt": col(b_rows, 3),
        "aptr": aptr, "ai": col(a_rows, 2), "aj": col(a_rows, 3), "at": col(a_rows, 4), "acen": col(a_rows, 5),
        "dptr": dptr, "di": col(d_rows, 2), "dj": col(d_rows, 3), "dl": col(d_rows, 4), "dt": col(d_rows, 5),
        "dcen": col(d_rows, 6),
    }
