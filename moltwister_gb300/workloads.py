"""Seeded synthetic systems for the benchmark configurations and the parity cases.

Units are the reference's (Cmd/MolTwisterCmdMolDyn/Integrators/Constants.h:23-40): A, g/mol, kJ/mol,
time unit 100 fs, kT = T[K] / 120.272, momentum p = m v with v in A/(100 fs).

Every generator takes an explicit seed and uses numpy's PCG64 generator, so the same call gives
the same system on any host.
"""
from __future__ import annotations

import math
from typing import Optional, Tuple

import numpy as np

from .system import (AngleTerm, BondTerm, DihedralTerm, MDConfig, MDSystem, NonBondedTerm)

CONV_T = 120.272          # K per (kJ/mol): Constants.h Conv_T
COULOMB_K = 1389.32       # Constants.h Coulomb_K (used as a float by the reference)

M_AR = 39.948
M_O, M_H = 15.999, 1.008
Q_O, Q_H = -0.8476, 0.4238


def maxwell_boltzmann(m: np.ndarray, T: float, rng: np.random.Generator,
                      mobile: Optional[np.ndarray] = None) -> np.ndarray:
    """Maxwell-Boltzmann momenta at T [K], centre-of-mass momentum removed, then rescaled so that
    the reference's temperature estimator sum(p^2/m)/(3N) (SimulationBox.cpp:168-180) equals kT."""
    kT = T / CONV_T
    p = rng.standard_normal((m.shape[0], 3)) * np.sqrt(m * kT)[:, None]
    if mobile is not None:
        p[~mobile] = 0.0
    mob = np.ones(m.shape[0], bool) if mobile is None else mobile
    if mob.sum() > 1:
        p[mob] -= p[mob].sum(axis=0) / mob.sum()
    t_now = float(np.sum(p * p / m[:, None]) / (3.0 * m.shape[0]))
    if t_now > 0:
        p *= math.sqrt(kT / t_now)
    return p


def nh_initial(M: int, N: int, T: float, tau_fs: float, rng: np.random.Generator) -> Tuple[np.ndarray, np.ndarray]:
    """Seeded Nose-Hoover chain state: eta uniform in [0,1) as CNHChain::setRandNHPos
    (NHChain.cpp:126-133), and thermal chain momenta p_eta_j ~ N(0, Q_j kT) with
    Q_0 = 3 N kT tau^2, Q_j = kT tau^2 (NHChain.cpp:115-124).

    The reference draws p_eta uniformly in [-Q_j/tau, Q_j/tau] (NHChain.cpp:135-143); with its
    Suzuki-Yoshida weights w0 = 1/(1 - 2^(1/3)) (NHChain.cpp:45-52) such starts can diverge within a
    few steps, so the seeded systems start from thermal chain momenta instead."""
    kT = T / CONV_T
    tau = tau_fs / 100.0
    Q = np.array([3.0 * N * kT * tau * tau] + [kT * tau * tau] * (M - 1))
    eta = rng.random(M)
    peta = rng.standard_normal(M) * np.sqrt(Q * kT)
    return eta, peta


def npt_initial(M: int, T: float, tauP_fs: float, rng: np.random.Generator):
    """Seeded barostat state: p_eps ~ N(0, W kT) with W = kT tauP^2 (SimulationBox.cpp:73), and the
    barostat chain as nh_initial with Q_0 = kT tauP^2 (prepareArrays(1, 1), SimulationBox.cpp:88)."""
    kT = T / CONV_T
    tau = tauP_fs / 100.0
    W = kT * tau * tau
    p_eps = float(rng.standard_normal() * np.sqrt(W * kT))
    Q = np.array([kT * tau * tau] * M)
    eta = rng.random(M)
    peta = rng.standard_normal(M) * np.sqrt(Q * kT)
    return p_eps, eta, peta


def make_npt(sys_: "MDSystem", cfg: "MDConfig", pressure_atm: float, seed: int):
    """Switches a seeded system to NPT at `pressure_atm` with a seeded barostat state."""
    cfg.ensemble = "NPT"
    cfg.pressure = pressure_atm
    rng = np.random.default_rng(seed)
    sys_.p_eps, sys_.nhP_eta, sys_.nhP_peta = npt_initial(cfg.pressurenhlen, cfg.temperature, cfg.pressurerelax, rng)
    return sys_, cfg


# ------------------------------------------------------------------------------------------------
# Config 1: LJ argon, FCC lattice, reduced density 0.8
# ------------------------------------------------------------------------------------------------
def fcc_positions(ncell: int, a: float) -> np.ndarray:
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.arange(ncell)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pos = (cells[:, None, :] + base[None, :, :]).reshape(-1, 3) * a
    L = ncell * a
    pos = pos - L / 2.0 + a / 4.0       # centred in [-L/2, L/2)
    return pos


def argon(ncell: int = 10, seed: int = 1, T: float = 120.0, rho_star: float = 0.8,
          sigma: float = 3.405, eps: float = 0.996, jitter: float = 0.0,
          charge: float = 0.0) -> Tuple[MDSystem, MDConfig]:
    """Config 1: LJ argon on an FCC lattice of ncell^3 cells (4 atoms each), cubic periodic box at
    reduced density rho_star, sigma=3.405 A, eps=0.996 kJ/mol, m=39.948, cutoff 2.5 sigma,
    Maxwell-Boltzmann momenta at T, Nose-Hoover at T, dt=2 fs."""
    rng = np.random.default_rng(seed)
    a = (4.0 / rho_star) ** (1.0 / 3.0) * sigma
    r = fcc_positions(ncell, a)
    if jitter > 0:
        r = r + rng.uniform(-jitter, jitter, r.shape)
    N = r.shape[0]
    L = ncell * a
    m = np.full(N, M_AR)
    sys_ = MDSystem(box=np.array([L, L, L]), ids=["Ar"] * N, r=r, q=np.full(N, charge), m=m,
                    mobile=np.ones(N, bool),
                    nonbonded=[NonBondedTerm("Ar", "Ar", "LJ", (eps, sigma))])
    sys_.mol = np.arange(N, dtype=np.int32)
    sys_.p = maxwell_boltzmann(m, T, rng)
    cfg = MDConfig(timestep=2.0, timesteps=1000, temperature=T, temperaturerelax=40.0,
                   cutoffradius=2.5 * sigma, neighshell=2.0, ensemble="NVT")
    sys_.nhT_eta, sys_.nhT_peta = nh_initial(cfg.temperaturenhlen, N, T, cfg.temperaturerelax, rng)
    return sys_, cfg


# ------------------------------------------------------------------------------------------------
# Config 3: Kob-Andersen binary LJ mixture (LJ reduced units with sigma = 1 A, eps = 1 kJ/mol,
# m = 1 g/mol: T* = 0.75 is 90.2 K, dt* = 0.005 is 0.5 fs)
# ------------------------------------------------------------------------------------------------
KA_PAIRS = {("A", "A"): (1.0, 1.0), ("A", "B"): (1.5, 0.8), ("B", "B"): (0.5, 0.88)}   # (eps, sigma)


def kob_andersen(ncell: int = 64, seed: int = 3, T_star: float = 0.75, rho_star: float = 1.2,
                 frac_a: float = 0.8, jitter: float = 0.05, per_pair_cutoff: bool = True,
                 dt_fs: float = 0.5, placement: str = "lattice") -> Tuple[MDSystem, MDConfig]:
    """Kob-Andersen 80:20 mixture, N = 4 ncell^3 (ncell = 64: 1,048,576 atoms) at reduced
    density rho_star, with a seeded random A/B assignment: placement "lattice" puts the atoms on
    FCC sites with seeded jitter, "random" uniformly at random in the box (seeded; overlapping
    atoms then need relax_random before dynamics).  eps/sigma AA 1/1, AB 1.5/0.8, BB 0.5/0.88,
    cutoff 2.5 sigma_ab per pair (with per_pair_cutoff; else 2.5 for every pair, the only form the
    reference can express), energies shifted to zero at the cutoffs, Maxwell-Boltzmann momenta at
    T*, NVE."""
    rng = np.random.default_rng(seed)
    a = (4.0 / rho_star) ** (1.0 / 3.0)
    r = fcc_positions(ncell, a)
    N = r.shape[0]
    if placement == "random":
        L = ncell * a
        r = rng.uniform(-0.5 * L, 0.5 * L, (N, 3))
    elif placement != "lattice":
        raise ValueError(placement)
    elif jitter > 0:
        r = r + rng.uniform(-jitter, jitter, r.shape)
    nb = int(round((1.0 - frac_a) * N))
    ids = np.array(["A"] * N, dtype=object)
    ids[rng.permutation(N)[:nb]] = "B"
    L = ncell * a
    m = np.ones(N)
    T = T_star * CONV_T
    terms = [NonBondedTerm(i, j, "LJ", (e, sg), cutoff=(2.5 * sg if per_pair_cutoff else 0.0))
             for (i, j), (e, sg) in KA_PAIRS.items()]
    sys_ = MDSystem(box=np.array([L, L, L]), ids=[str(x) for x in ids], r=r, q=np.zeros(N), m=m,
                    mobile=np.ones(N, bool), nonbonded=terms)
    sys_.mol = np.arange(N, dtype=np.int32)
    sys_.p = maxwell_boltzmann(m, T, rng)
    cfg = MDConfig(timestep=dt_fs, timesteps=20000, temperature=T, ensemble="NVE",
                   cutoffradius=2.5, neighshell=0.3, listskin=0.3, coulomb="cutoff", coulombcutoff=2.5,
                   precision="mixed", ljshift=True, clipforces=False, optlearningrate=1e-4)
    return sys_, cfg


# Learning-rate stages of relax_random: the mixed force gather caps every pair force at about
# 2.6e5 (its fixed-point range), so the first stages move overlapping atoms by at most a few
# hundredths of sigma per step while they separate; the later ones relax the structure.
RANDOM_RELAX_STAGES = ((1e-7, 100), (1e-6, 100), (1e-5, 200), (1e-4, 200))


def relax_random(s: "MDSystem", cfg: "MDConfig", stages=RANDOM_RELAX_STAGES, device: int = 0) -> np.ndarray:
    """Gradient descent (Engine.optimize, the reference's optimizeenergy) from a random placement,
    in stages of growing learning rate, in the mixed mode; returns the relaxed positions."""
    from .engine import Engine
    from .system import MDConfig as _C
    r = np.array(s.r, np.float64)
    for lr, steps in stages:
        c = _C(**{k: getattr(cfg, k) for k in cfg.__dataclass_fields__})
        c.precision = "mixed"
        c.optlearningrate = lr
        si = s.copy()
        si.r = r
        e = Engine(si, c, device=device)
        e.optimize(steps)
        r = e.get_state()[0]
        e.close()
    return r


# ------------------------------------------------------------------------------------------------
# Config 5: ensembles of argon and water replicas of uneven size
# ------------------------------------------------------------------------------------------------
ARGON_RC = 2.5 * 3.405


def argon_n(n: int, seed: int, T: float, rho_star: float = 0.8, sigma: float = 3.405, eps: float = 0.996,
            jitter: float = 0.05) -> Tuple[MDSystem, MDConfig]:
    """LJ argon with exactly n atoms at reduced density rho_star: n sites drawn (seeded) from the
    smallest simple cubic lattice with at least n sites in the box, jittered; the LJ term carries
    its own cutoff 2.5 sigma."""
    rng = np.random.default_rng(seed)
    L = (n / rho_star) ** (1.0 / 3.0) * sigma
    m = int(math.ceil(n ** (1.0 / 3.0) - 1e-9))
    a = L / m
    g = np.arange(m)
    sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) * a - L / 2.0 + a / 2.0
    r = sites[rng.permutation(sites.shape[0])[:n]] + rng.uniform(-jitter, jitter, (n, 3))
    mass = np.full(n, M_AR)
    sys_ = MDSystem(box=np.array([L, L, L]), ids=["Ar"] * n, r=r, q=np.zeros(n), m=mass, mobile=np.ones(n, bool),
                    nonbonded=[NonBondedTerm("Ar", "Ar", "LJ", (eps, sigma), cutoff=ARGON_RC)])
    sys_.mol = np.arange(n, dtype=np.int32)
    sys_.p = maxwell_boltzmann(mass, T, rng)
    cfg = MDConfig(timestep=0.5, temperature=T, temperaturerelax=20.0, cutoffradius=ARGON_RC, ensemble="NVT")
    sys_.nhT_eta, sys_.nhT_peta = nh_initial(cfg.temperaturenhlen, n, T, cfg.temperaturerelax, rng)
    return sys_, cfg


def replica_spec(nrep: int = 512, seed: int = 5, nmin: int = 200, nmax: int = 20000,
                 tmin: float = 80.0, tmax: float = 400.0):
    """[(kind, n_atoms, T, seed)] of a seeded replica ensemble: kind 'argon' or 'water' by seed,
    sizes uniform in [nmin, nmax] (water rounded down to whole molecules), temperatures uniform in
    [tmin, tmax] K."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(nrep):
        kind = "argon" if rng.random() < 0.5 else "water"
        n = int(rng.integers(nmin, nmax + 1))
        if kind == "water":
            n = max(3 * (n // 3), 3 * ((nmin + 2) // 3))
        out.append((kind, n, float(rng.uniform(tmin, tmax)), int(rng.integers(1 << 30))))
    return out


def make_replica(kind: str, n: int, T: float, seed: int, rc_max: float = 10.0):
    """(system, pair cutoff) of one replica: argon (LJ cutoff 2.5 sigma) or water (cutoff rc_max),
    the cutoff shortened to below half the box when the box is small."""
    if kind == "argon":
        s, _ = argon_n(n, seed, T)
        rc = ARGON_RC
    else:
        nm = n // 3
        s, _ = water(n_mol=nm, L=water_box_length(nm), seed=seed, T=T, rc=rc_max)
        rc = rc_max
    return s, min(rc, 0.5 * float(s.box.min()) - 0.05)


# ------------------------------------------------------------------------------------------------
# Config 2: flexible SPC/E-like water
# ------------------------------------------------------------------------------------------------
def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water(n_mol: int = 3000, L: float = 44.8, seed: int = 2, T: float = 300.0,
          r0: float = 1.0, theta0: float = 109.47, lattice: Optional[int] = None,
          rc: float = 10.0, dt: float = 0.5, min_contact: float = 1.8) -> Tuple[MDSystem, MDConfig]:
    """Config 2: flexible SPC/E-like water.  Molecules on a seeded cubic lattice (lattice^3 sites,
    the first n_mol of a seeded permutation), random orientations redrawn until no atom lies within
    min_contact of a neighbouring molecule (hydrogens carry no repulsive core).  Harmonic O-H bonds
    (r0=1.0 A, k=4637), harmonic H-O-H angle (theta0=109.47 deg, k=383) in the reference convention
    U = k (x - x0)^2, LJ on O-O only (sigma=3.166 A, eps=0.650), qO=-0.8476, qH=+0.4238."""
    rng = np.random.default_rng(seed)
    if lattice is None:
        lattice = int(math.ceil(n_mol ** (1.0 / 3.0) - 1e-9))
    spacing = L / lattice
    g = np.arange(lattice)
    grid = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    grid = grid[rng.permutation(grid.shape[0])[:n_mol]]
    sites = grid * spacing - L / 2.0 + spacing / 2.0
    th = math.radians(theta0) / 2.0
    h1 = np.array([r0 * math.sin(th), r0 * math.cos(th), 0.0])
    h2 = np.array([-r0 * math.sin(th), r0 * math.cos(th), 0.0])
    N = 3 * n_mol
    r = np.zeros((N, 3))
    ids, q, m = [], np.zeros(N), np.zeros(N)
    bonds, angles = [], []
    placed = {}
    offsets = [(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1) if (a, b, c) != (0, 0, 0)]
    for i in range(n_mol):
        o = sites[i]
        key = tuple(int(v) for v in grid[i])
        near = [placed[k2] for k2 in (tuple((key[a] + off[a]) % lattice for a in range(3)) for off in offsets)
                if k2 in placed]
        near = np.concatenate(near) if near else np.zeros((0, 3))
        # random orientation, redrawn (at most 60 times) until no atom comes within min_contact of
        # an already placed molecule; the best draw is kept otherwise
        best, best_d = None, -1.0
        for _ in range(60):
            R = random_rotation(rng)
            mol3 = np.stack([o, o + R @ h1, o + R @ h2])
            if near.shape[0] == 0:
                best = mol3
                break
            dd = mol3[:, None, :] - near[None, :, :]
            dd -= L * np.rint(dd / L)
            dmin = float(np.sqrt((dd * dd).sum(-1).min()))
            if dmin > best_d:
                best, best_d = mol3, dmin
            if dmin >= min_contact:
                break
        r[3 * i:3 * i + 3] = best
        placed[key] = best
        ids += ["Ow", "Hw", "Hw"]
        q[3 * i:3 * i + 3] = (Q_O, Q_H, Q_H)
        m[3 * i:3 * i + 3] = (M_O, M_H, M_H)
        bonds += [(3 * i, 3 * i + 1, 0), (3 * i, 3 * i + 2, 0)]
        angles += [(3 * i + 1, 3 * i, 3 * i + 2, 0)]
    # keep atoms inside [-L/2, L/2)
    r = r - L * np.floor((r + L / 2.0) / L)
    sys_ = MDSystem(box=np.array([L, L, L]), ids=ids, r=r, q=q, m=m, mobile=np.ones(N, bool),
                    nonbonded=[NonBondedTerm("Ow", "Ow", "LJ", (0.650, 3.166))],
                    bond_terms=[BondTerm("Ow", "Hw", "Harm", (4637.0, r0), "all_r_less_than", 1.1)],
                    angle_terms=[AngleTerm("Hw", "Ow", "Hw", "Harm", (383.0, theta0), "all_r_less_than", 1.1)])
    sys_.bonds = np.array(bonds, np.int32).reshape(-1, 3)
    sys_.angles = np.array(angles, np.int32).reshape(-1, 4)
    sys_.mol = np.repeat(np.arange(n_mol, dtype=np.int32), 3)
    sys_.p = maxwell_boltzmann(m, T, rng)
    cfg = MDConfig(timestep=dt, timesteps=10000, temperature=T, temperaturerelax=20.0 * dt,
                   cutoffradius=rc, neighshell=2.0, ensemble="NVT", scale12=0.0, scale13=0.0)
    sys_.nhT_eta, sys_.nhT_peta = nh_initial(cfg.temperaturenhlen, N, T, cfg.temperaturerelax, rng)
    return sys_, cfg


def water_box_length(n_mol: int, density_g_cm3: float = 1.0) -> float:
    """Cubic box edge [A] holding n_mol waters at the given mass density."""
    mass_g = n_mol * (M_O + 2 * M_H) / 6.02214076e23
    vol_A3 = mass_g / density_g_cm3 * 1e24
    return vol_A3 ** (1.0 / 3.0)


# ------------------------------------------------------------------------------------------------
# Small mixed-topology case: chains with bonds, angles and dihedrals, Buckingham + LJ + charges
# ------------------------------------------------------------------------------------------------
def chains(n_chain: int = 27, L: float = 24.0, seed: int = 5, T: float = 250.0,
           immobile_every: int = 0) -> Tuple[MDSystem, MDConfig]:
    """Four-atom chains C1-C2-C3-C4 on a seeded lattice, random orientation, with harmonic bonds,
    harmonic angles, a harmonic dihedral on C1-C2-C3-C4 and a Fourier4t dihedral added on the same
    quadruple through a second term type; Buckingham between end atoms, LJ elsewhere, small
    charges.  Exercises every term kind the reference tabulates except Class2/LJ1208/LJBuck."""
    rng = np.random.default_rng(seed)
    lattice = int(math.ceil(n_chain ** (1.0 / 3.0) - 1e-9))
    spacing = L / lattice
    g = np.arange(lattice)
    sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) * spacing - L / 2.0 + spacing / 2.0
    sites = sites[rng.permutation(sites.shape[0])[:n_chain]]
    b = 1.53
    ang = math.radians(112.0)
    phi = math.radians(65.0)
    c1 = np.array([0.0, 0.0, 0.0])
    c2 = np.array([b, 0.0, 0.0])
    c3 = c2 + b * np.array([-math.cos(ang), math.sin(ang), 0.0])
    u = (c3 - c2) / b                                  # bond axis C2->C3
    t = c1 - c2
    t = t - np.dot(t, u) * u
    t /= np.linalg.norm(t)                             # in-plane normal, towards C1 (cis side)
    z = np.cross(u, t)
    c4 = c3 + b * (-math.cos(ang) * u + math.sin(ang) * (math.cos(phi) * t + math.sin(phi) * z))
    local = np.vstack([c1, c2, c3, c4])
    local -= local.mean(axis=0)
    N = 4 * n_chain
    r = np.zeros((N, 3))
    ids, q, m = [], np.zeros(N), np.zeros(N)
    bonds, angles, dihs = [], [], []
    for i in range(n_chain):
        R = random_rotation(rng)
        for j in range(4):
            r[4 * i + j] = sites[i] + R @ local[j]
        ids += ["Ce", "Cm", "Cm", "Ce"]
        q[4 * i:4 * i + 4] = (0.12, -0.12, -0.12, 0.12)
        m[4 * i:4 * i + 4] = (15.035, 14.027, 14.027, 15.035)
        k = 4 * i
        bonds += [(k, k + 1, 0), (k + 1, k + 2, 1), (k + 2, k + 3, 0)]
        angles += [(k, k + 1, k + 2, 0), (k + 1, k + 2, k + 3, 0)]
        dihs += [(k, k + 1, k + 2, k + 3, 0)]
    r = r - L * np.floor((r + L / 2.0) / L)
    mobile = np.ones(N, bool)
    if immobile_every:
        mobile[::immobile_every] = False
    sys_ = MDSystem(
        box=np.array([L, L, L]), ids=ids, r=r, q=q, m=m, mobile=mobile,
        nonbonded=[NonBondedTerm("Ce", "Ce", "Buck", (50000.0, 0.30, 2000.0)),
                   NonBondedTerm("Ce", "Cm", "LJ", (0.60, 3.8)),
                   NonBondedTerm("Cm", "Cm", "LJ", (0.40, 3.9, 0.9)),
                   NonBondedTerm("Ce", "Ce", "LJ", (0.05, 3.0))],
        bond_terms=[BondTerm("Ce", "Cm", "Harm", (1300.0, 1.53), "all_r_less_than", 1.8),
                    BondTerm("Cm", "Cm", "Morse", (350.0, 1.9, 1.53), "all_r_less_than", 1.8)],
        angle_terms=[AngleTerm("Ce", "Cm", "Cm", "Harm", (260.0, 112.0), "all_r_less_than", 1.8)],
        dihedral_terms=[DihedralTerm("Ce", "Cm", "Cm", "Ce", "Harm", (5.0, 1.0, 3.0), "all_r_less_than", 1.8)])
    sys_.bonds = np.array(bonds, np.int32).reshape(-1, 3)
    sys_.angles = np.array(angles, np.int32).reshape(-1, 4)
    sys_.dihedrals = np.array(dihs, np.int32).reshape(-1, 5)
    sys_.mol = np.repeat(np.arange(n_chain, dtype=np.int32), 4)
    sys_.p = maxwell_boltzmann(m, T, rng, mobile)
    cfg = MDConfig(timestep=1.0, timesteps=100, temperature=T, temperaturerelax=20.0,
                   cutoffradius=7.5, neighshell=0.4, ensemble="NVT", scale14=0.5)
    sys_.nhT_eta, sys_.nhT_peta = nh_initial(cfg.temperaturenhlen, N, T, cfg.temperaturerelax, rng)
    return sys_, cfg
