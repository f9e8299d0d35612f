"""TEST INFRASTRUCTURE: an FP64 reference adjoint for the pair-correlation trajectory loss, in
numpy, independent of the CUDA library.  Only tests/ use it.

Model (the flexible-water terms of the benchmark): 12-6 LJ per type pair (a = 4 eps sigma^12,
b = 4 eps sigma^6) and shifted-force Coulomb (K = 1389.32, cutoff rc) over all pairs of different
molecules within rc (minimum image), harmonic bonds U = k (r - r0)^2 and harmonic angles
U = k (theta - theta0)^2 (the reference's conventions, MolTwisterMDFFBond_Harm.cpp:90-110,
MolTwisterMDFFAngle_Harm.cpp:94-130).  Trajectory: plain velocity Verlet.  Loss: squared deviation
of the Gaussian-smeared pair correlation of two types averaged over the positions after each step
(the definition of mtg_loss_grad in include/mtgpu.h).

Force tangents (Hessian-vector products and parameter derivatives of the forces) use forward-mode
dual numbers over numpy arrays; the backward pass is the leapfrog adjoint of velocity Verlet.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

KC = 1389.32


class D:
    """Dual array v + t eps."""
    __slots__ = ("v", "t")

    def __init__(self, v, t=None):
        self.v = np.asarray(v, np.float64)
        self.t = np.zeros_like(self.v) if t is None else np.asarray(t, np.float64)

    def __add__(self, o):
        o = o if isinstance(o, D) else D(o)
        return D(self.v + o.v, self.t + o.t)

    __radd__ = __add__

    def __sub__(self, o):
        o = o if isinstance(o, D) else D(o)
        return D(self.v - o.v, self.t - o.t)

    def __rsub__(self, o):
        return D(o) - self

    def __neg__(self):
        return D(-self.v, -self.t)

    def __mul__(self, o):
        o = o if isinstance(o, D) else D(o)
        return D(self.v * o.v, self.t * o.v + self.v * o.t)

    __rmul__ = __mul__

    def __truediv__(self, o):
        o = o if isinstance(o, D) else D(o)
        return D(self.v / o.v, (self.t * o.v - self.v * o.t) / (o.v * o.v))

    def __rtruediv__(self, o):
        return D(o) / self

    def __getitem__(self, k):
        return D(self.v[k], self.t[k])


def dsqrt(a: D) -> D:
    s = np.sqrt(a.v)
    return D(s, a.t * 0.5 / s)


def dacos(a: D) -> D:
    c = np.clip(a.v, -1.0, 1.0)
    s = np.maximum(np.sqrt(1.0 - c * c), 1e-6)
    return D(np.arccos(c), -a.t / s)


@dataclass
class Model:
    box: np.ndarray
    m: np.ndarray
    types: np.ndarray
    mol: np.ndarray
    dq: np.ndarray                       # charge direction: q = theta_q * dq
    lj: Dict[Tuple[int, int], Tuple[float, float]]   # (ta, tb) -> (eps, sigma), symmetric
    bonds: np.ndarray                    # (nb, 2) atom pairs
    angles: np.ndarray                   # (na, 3) (a1, centre, a3)
    rc: float
    lj_force_shift: bool = False         # LJ force and energy shifted at rc (continuous forces)
    # parameters: eps, sigma (of lj_pair), q (theta_q), bond k, bond r0, angle k, angle theta0 [deg]
    lj_pair: Tuple[int, int] = (0, 0)
    theta: Dict[str, float] = field(default_factory=dict)
    pairs: Optional[np.ndarray] = None

    def __post_init__(self):
        n = len(self.m)
        i, j = np.triu_indices(n, 1)
        keep = self.mol[i] != self.mol[j]
        self.pairs = np.stack([i[keep], j[keep]], 1)


def _minimg(d: np.ndarray, L: np.ndarray) -> np.ndarray:
    return d - L * np.rint(d / L)


def forces(M: Model, r: np.ndarray, vr: Optional[np.ndarray] = None, tan: Optional[str] = None) -> Tuple[D, D]:
    """(F, U) as dual numbers: tangent along positions vr, or along parameter `tan`."""
    n = len(M.m)
    th = {k: D(v, 1.0 if k == tan else 0.0) for k, v in M.theta.items()}
    vr = np.zeros_like(r) if vr is None else vr
    F = [D(np.zeros(n)) for _ in range(3)]
    U = D(0.0)

    def add(idx, comp, val: D):
        F[comp] = D(F[comp].v + np.bincount(idx, val.v, n), F[comp].t + np.bincount(idx, val.t, n))

    # pairs
    i, j = M.pairs[:, 0], M.pairs[:, 1]
    dv = _minimg(r[i] - r[j], M.box)
    dt = vr[i] - vr[j]
    dd = [D(dv[:, a], dt[:, a]) for a in range(3)]
    r2 = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]
    sel = r2.v < M.rc * M.rc
    i, j = i[sel], j[sel]
    dd = [x[sel] for x in dd]
    r2 = r2[sel]
    rr = dsqrt(r2)
    ir = 1.0 / rr
    ir2 = ir * ir
    g = D(np.zeros(len(i)))
    u = D(np.zeros(len(i)))
    lj_mask = np.zeros(len(i), bool)
    for (ta, tb), (e0, s0) in M.lj.items():
        mk = ((M.types[i] == ta) & (M.types[j] == tb)) | ((M.types[i] == tb) & (M.types[j] == ta))
        if ta != tb:
            pass
        mk &= ~lj_mask
        lj_mask |= mk
        if not mk.any():
            continue
        if (ta, tb) == M.lj_pair or (tb, ta) == M.lj_pair:
            eps, sig = th["eps"], th["sigma"]
        else:
            eps, sig = D(e0), D(s0)
        s2 = sig * sig
        s6 = s2 * s2 * s2
        a = 4.0 * eps * s6 * s6
        b = 4.0 * eps * s6
        ir6 = ir2[mk] * ir2[mk] * ir2[mk]
        t12 = a * ir6 * ir6
        t6 = b * ir6
        gk = (12.0 * t12 - 6.0 * t6) * ir2[mk]
        uk = t12 - t6
        if M.lj_force_shift:
            c6 = 1.0 / M.rc ** 6
            Uc = a * (c6 * c6) - b * c6
            Fc = (12.0 * a * (c6 * c6) - 6.0 * b * c6) / M.rc
            gk = gk - Fc * ir[mk]
            uk = uk - Uc + (rr[mk] - M.rc) * Fc
        g = D(g.v.copy(), g.t.copy())
        g.v[mk] += gk.v
        g.t[mk] += gk.t
        u.v[mk] += uk.v
        u.t[mk] += uk.t
    q = th["q"]
    qq = KC * (q * q) * D(M.dq[i] * M.dq[j])
    irc = 1.0 / M.rc
    gc = qq * (ir2 - irc * irc) * ir
    uc = qq * (ir - irc + (rr - M.rc) * (irc * irc))
    g = g + gc
    u = u + uc
    for a in range(3):
        f = g * dd[a]
        add(i, a, f)
        add(j, a, -f)
    U = U + D(u.v.sum(), u.t.sum())
    # bonds
    if len(M.bonds):
        i, j = M.bonds[:, 0], M.bonds[:, 1]
        dv = _minimg(r[i] - r[j], M.box)
        dt = vr[i] - vr[j]
        dd = [D(dv[:, a], dt[:, a]) for a in range(3)]
        rr = dsqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2])
        k, r0 = th["bond_k"], th["bond_r0"]
        dr = rr - r0
        md = -2.0 * k * dr
        s = md / rr
        for a in range(3):
            f = s * dd[a]
            add(i, a, f)
            add(j, a, -f)
        ub = k * dr * dr
        U = U + D(ub.v.sum(), ub.t.sum())
    # angles
    if len(M.angles):
        a1, c, a3 = M.angles[:, 0], M.angles[:, 1], M.angles[:, 2]
        uvv = _minimg(r[a1] - r[c], M.box)
        vvv = _minimg(r[a3] - r[c], M.box)
        ut = vr[a1] - vr[c]
        vt = vr[a3] - vr[c]
        uu = [D(uvv[:, x], ut[:, x]) for x in range(3)]
        vv = [D(vvv[:, x], vt[:, x]) for x in range(3)]
        n1 = dsqrt(uu[0] * uu[0] + uu[1] * uu[1] + uu[2] * uu[2])
        n3 = dsqrt(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2])
        cs = (uu[0] * vv[0] + uu[1] * vv[1] + uu[2] * vv[2]) / (n1 * n3)
        tha = dacos(cs)
        sn = dsqrt(1.0 - cs * cs)
        sn = D(np.maximum(sn.v, 1e-6), np.where(sn.v < 1e-6, 0.0, sn.t))
        k, t0 = th["angle_k"], th["angle_theta0"] * (np.pi / 180.0)
        dU = 2.0 * k * (tha - t0)
        inv = 1.0 / (n1 * n3)
        for x in range(3):
            g1 = -(vv[x] * inv - cs * uu[x] / (n1 * n1)) / sn
            g3 = -(uu[x] * inv - cs * vv[x] / (n3 * n3)) / sn
            f1 = -dU * g1
            f3 = -dU * g3
            add(a1, x, f1)
            add(a3, x, f3)
            add(c, x, -(f1 + f3))
        ua = k * (tha - t0) * (tha - t0)
        U = U + D(ua.v.sum(), ua.t.sum())
    Fv = np.stack([F[a].v for a in range(3)], 1)
    Ft = np.stack([F[a].t for a in range(3)], 1)
    return D(Fv, Ft), U


def rdf_frame(M: Model, r: np.ndarray, ta: int, tb: int, nbins: int, rmax: float, width: float,
              cb: Optional[np.ndarray] = None):
    """Smeared pair histogram sum_pairs K(r_ij - x_b) of one frame, and (with cb) the position
    gradient of sum_b cb_b * histogram_b."""
    dr = rmax / nbins
    x = (np.arange(nbins) + 0.5) * dr
    ia = np.where(M.types == ta)[0]
    ib = np.where(M.types == tb)[0]
    if ta == tb:
        i, j = np.triu_indices(len(ia), 1)
        i, j = ia[i], ia[j]
    else:
        i, j = np.repeat(ia, len(ib)), np.tile(ib, len(ia))
    keep = M.mol[i] != M.mol[j]
    i, j = i[keep], j[keep]
    d = _minimg(r[i] - r[j], M.box)
    rr = np.sqrt((d * d).sum(1))
    near = rr <= rmax + 8.0 * width
    i, j, d, rr = i[near], j[near], d[near], rr[near]
    z = rr[:, None] - x[None, :]
    win = np.abs(z) <= 8.0 * width
    K = np.where(win, np.exp(-0.5 * (z / width) ** 2) / (width * np.sqrt(2.0 * np.pi)), 0.0)
    hist = K.sum(0)
    if cb is None:
        return hist, None
    dK = K * (-z / width ** 2)
    s = (dK * cb[None, :]).sum(1) / rr
    g = np.zeros_like(r)
    for a in range(3):
        g[:, a] += np.bincount(i, s * d[:, a], len(r))
        g[:, a] -= np.bincount(j, s * d[:, a], len(r))
    return hist, g


def loss_and_grad(M: Model, r0: np.ndarray, p0: np.ndarray, dt: float, nsteps: int, ta: int, tb: int, nbins: int,
                  rmax: float, width: float, target: np.ndarray, names: List[str], adjoint: bool = True):
    """(L, dL/dtheta for `names`, gbar) by the leapfrog adjoint of velocity Verlet."""
    n = len(M.m)
    im = (1.0 / M.m)[:, None]
    rs = [r0.copy()]
    r = r0.copy()
    F, _ = forces(M, r)
    v = p0 + 0.5 * dt * F.v
    hsum = np.zeros(nbins)
    for t in range(nsteps):
        r = r + dt * v * im
        rs.append(r.copy())
        F, _ = forces(M, r)
        v = v + dt * F.v
        hsum += rdf_frame(M, r, ta, tb, nbins, rmax, width)[0]
    na = int((M.types == ta).sum())
    nb = int((M.types == tb).sum())
    npairs = 0.5 * na * (na - 1) if ta == tb else na * nb
    V = float(np.prod(M.box))
    x = (np.arange(nbins) + 0.5) * (rmax / nbins)
    norm = V / (npairs * 4.0 * np.pi * x * x)
    gbar = norm * hsum / nsteps
    dev = gbar - target
    L = float((dev * dev).sum())
    if not adjoint:
        return L, None, gbar
    cb = 2.0 * dev / nsteps * norm
    grad = np.zeros(len(names))
    lam_r = rdf_frame(M, rs[nsteps], ta, tb, nbins, rmax, width, cb)[1]
    lam_v = np.zeros_like(r0)
    for t in range(nsteps, 0, -1):
        lam_v = lam_v + dt * lam_r * im
        w = dt if t - 1 >= 1 else 0.5 * dt
        Fj, _ = forces(M, rs[t - 1], vr=lam_v)
        lam_r = lam_r + w * Fj.t
        for k, nm in enumerate(names):
            Fp, _ = forces(M, rs[t - 1], tan=nm)
            grad[k] += w * float((lam_v * Fp.t).sum())
        if t - 1 >= 1:
            lam_r = lam_r + rdf_frame(M, rs[t - 1], ta, tb, nbins, rmax, width, cb)[1]
    return L, grad, gbar


def water_model(s, rc: float, q_dir: Dict[str, float], lj_force_shift: bool = False) -> Model:
    """Model of a seeded water MDSystem (moltwister_gb300.workloads.water) with its parameters."""
    names = s.type_names()
    types = s.type_index()
    lj = {}
    for t in s.nonbonded:
        if t.kind == "LJ":
            lj[(names.index(t.id1), names.index(t.id2))] = (float(t.args[0]), float(t.args[1]))
    (pa, (e0, s0)), = lj.items()
    dq = np.array([q_dir.get(nm, 0.0) for nm in s.ids], np.float64)
    qO = float(s.q[np.nonzero(dq)[0][0]] / dq[np.nonzero(dq)[0][0]])
    bt = s.bond_terms[0]
    at = s.angle_terms[0]
    M = Model(box=np.asarray(s.box, np.float64), m=np.asarray(s.m, np.float64), types=types, mol=s.mol_index(), dq=dq,
              lj=lj, bonds=np.asarray(s.bonds)[:, :2].astype(int), angles=np.asarray(s.angles)[:, [0, 1, 2]].astype(int),
              rc=rc, lj_force_shift=lj_force_shift, lj_pair=pa,
              theta={"eps": e0, "sigma": s0, "q": qO, "bond_k": float(bt.args[0]), "bond_r0": float(bt.args[1]),
                     "angle_k": float(at.args[0]), "angle_theta0": float(at.args[1])})
    return M
