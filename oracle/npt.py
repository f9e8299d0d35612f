"""FP64 oracle of the production-mode NPT step (test infrastructure).

The production modes run the reference's MTK barostat and Nose-Hoover chains with four
differences, each a correction of the reference's arithmetic:
  - the barostat is driven by the pair virial sum_{i<j} r_ij . F_ij plus the bonded terms' virial
    (the reference sums F . r over wrapped positions, VelVerlet.cpp:160-174, which depends on where
    the box boundary cuts the molecules);
  - the chains use the published Suzuki-Yoshida weight w0 = 1/(2 - 2^(1/3)) and the exponential
    itself, without the p_eta[0] clamp (the reference: NHChain.cpp:45-52, 61-65, Math.cpp:29-38);
  - the prop_p / prop_r coefficients (VelVerlet.cpp:124-150) use the exponential itself;
  - the barostat mass is MTK's (N_f + 3) kT tauP^2 with N_f = 3N (the reference: kT tauP^2,
    SimulationBox.cpp:73-76, under which the volume oscillates about sqrt(3N) times faster than
    tauP); the barostat chain keeps the reference's masses kT tauP^2.
The step order is the reference's (MDLoop.cpp:128-133 with VelVerlet.cpp:57-71): barostat and
particle chains, half kick of p_eps (3.1), prop_p (3.2), prop_r (3.3), strain and box (3.4),
forces, prop_p (3.5), half kick of p_eps (3.6), chains, pbcWrap.  Forces, energies and virials
come from the C oracle (orc_forces_fp64_vir: all pairs within the cutoffs, minimum image); the
loop runs in Python, so keep the systems small.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from moltwister_gb300.system import MDConfig, MDSystem

from .oracle import CONV_PRESS, CONV_T, Oracle, _p, lib


def _forces(orc: Oracle, box):
    n = orc.s.n
    for a in range(3):
        orc.st.box[a] = float(box[a])
    F = np.zeros((n, 3))
    U = np.zeros(n)
    W = np.zeros(n)
    rcut = float(orc.cfg.cutoffradius)
    lib().orc_forces_fp64_vir(C.byref(orc.st), rcut, _p(F), _p(U), _p(W))
    return F, U, W


def _sinhx_over_x(x: float) -> float:
    a = (1.0, 1.0 / 6.0, 1.0 / 120.0, 1.0 / 5040.0, 1.0 / 362880.0, 1.0 / 39916800.0)
    s, xn = 0.0, 1.0
    for c in a:
        s += c * xn
        xn *= x * x
    return s


def _chain_half(pe, eta, Q, KE2, g, kT, dt, nresp):
    """One propagator call (NHChain.cpp:54-113) on a driven kinetic term KE2 (sum p^2/m, or
    p_eps^2/W for the barostat) with the published weights; returns the momentum scale."""
    M = len(pe)
    w0 = 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))
    w = (w0, 1.0 - 2.0 * w0, w0)
    scale = 1.0

    def G(j):
        if j == 0:
            return KE2 * scale * scale - g * kT
        return pe[j - 1] * pe[j - 1] / Q[j - 1] - kT

    for mu in range(3):
        Dt = w[mu] * dt / nresp
        for _ in range(nresp):
            pe[M - 1] += (Dt / 4.0) * G(M - 1)
            for j in range(M - 1):
                co = np.exp(-(Dt / 8.0) * (pe[j + 1] / Q[j + 1]))
                pe[j] = (pe[j] * co + (Dt / 4.0) * G(j)) * co
            for j in range(M):
                eta[j] += (Dt / 2.0) * (pe[j] / Q[j])
            scale *= np.exp(-(Dt / 2.0) * (pe[0] / Q[0]))
            for j in range(M - 2, -1, -1):
                co = np.exp(-(Dt / 8.0) * (pe[j + 1] / Q[j + 1]))
                pe[j] = (pe[j] * co + (Dt / 4.0) * G(j)) * co
            pe[M - 1] += (Dt / 4.0) * G(M - 1)
    return scale


def run_npt(s: MDSystem, cfg: MDConfig, nsteps: int, stride: int):
    """Production NPT from the system's state (positions, momenta, chain states, p_eps; strain 0).
    Returns the records [(step, r, p, U, K, T, P, V, H)] at step 0 and every `stride` steps (H the
    extended energy the MTK equations conserve), and the
    final state dict (r, p, eta, peta, p_eps, eps, etaP, petaP, box)."""
    orc = Oracle(s, cfg)
    n = s.n
    m = np.asarray(s.m, np.float64)[:, None]
    r = np.array(s.r, np.float64)
    p = np.array(s.p, np.float64)
    dt = cfg.timestep / 100.0
    kT = cfg.temperature / CONV_T
    tau = cfg.temperaturerelax / 100.0
    tauP = cfg.pressurerelax / 100.0
    Pext = cfg.pressure / CONV_PRESS
    M, MP = cfg.temperaturenhlen, cfg.pressurenhlen
    Q = np.full(M, kT * tau * tau)
    Q[0] = 3.0 * n * kT * tau * tau
    QP = np.full(MP, kT * tauP * tauP)
    W = 3.0 * (n + 1.0) * kT * tauP * tauP      # MTK barostat mass (N_f + 3) kT tauP^2
    eta = np.array(s.nhT_eta if s.nhT_eta is not None else np.zeros(M), np.float64)
    peta = np.array(s.nhT_peta if s.nhT_peta is not None else np.zeros(M), np.float64)
    etaP = np.array(s.nhP_eta if s.nhP_eta is not None else np.zeros(MP), np.float64)
    petaP = np.array(s.nhP_peta if s.nhP_peta is not None else np.zeros(MP), np.float64)
    p_eps = float(s.p_eps) if s.p_eps is not None else 0.0
    eps = 0.0
    Lmax = np.array(s.box, np.float64)
    V0 = float(np.prod(Lmax))
    alpha = 1.0 + 1.0 / n
    box = Lmax.copy()

    def ke2():
        return float((p * p / m).sum())

    def wrap(x, L):
        h = L / 2.0
        x = np.where(x >= h, x - np.trunc((x + h) / L) * L, x)
        return np.where(x < -h, x - np.trunc((x - h) / L) * L, x)

    orc.r[...] = r
    F, U, Wv = _forces(orc, box)
    recs = []

    def record(step):
        K2 = ke2()
        V = V0 * np.exp(3.0 * eps)
        # the MTK extended energy: kinetic and potential energy, barostat kinetic energy, P V, and
        # both chains' kinetic and potential terms (conserved by the exact flow)
        H = (float(U.sum()) + 0.5 * K2 + p_eps * p_eps / (2.0 * W) + Pext * V
             + float((peta * peta / (2.0 * Q)).sum()) + 3.0 * n * kT * eta[0] + kT * float(eta[1:].sum())
             + float((petaP * petaP / (2.0 * QP)).sum()) + kT * float(etaP.sum()))
        recs.append((step, r.copy(), p.copy(), float(U.sum()), 0.5 * K2, K2 / (3.0 * n),
                     (K2 + float(Wv.sum())) / (3.0 * V), V, H))

    record(0)
    for t in range(nsteps):
        # barostat chain, particle chain (first halves), 3.1
        c = _chain_half(petaP, etaP, QP, p_eps * p_eps / W, 1.0, kT, dt, cfg.pressurerespa)
        p_eps *= c
        p *= _chain_half(peta, eta, Q, ke2(), 3.0 * n, kT, dt, cfg.temperaturerespa)
        V = V0 * np.exp(3.0 * eps)
        p_eps += (dt / 2.0) * (alpha * ke2() + float(Wv.sum()) - 3.0 * Pext * V)
        u = p_eps / W
        parm = alpha * u * dt / 4.0
        co = np.exp(-parm)
        ap, bp = co * co, (dt / 2.0) * co * _sinhx_over_x(parm)
        parm = u * dt / 2.0
        co = np.exp(parm)
        ar, br = co * co, dt * (_sinhx_over_x(parm) * co)
        p = p * ap + F * bp                                     # 3.2
        r = r * ar + (p / m) * br                               # 3.3
        eps += dt * p_eps / W                                   # 3.4
        ec = (V0 * np.exp(3.0 * eps) / float(np.prod(Lmax))) ** (1.0 / 3.0)
        box = ec * Lmax
        orc.r[...] = r
        F, U, Wv = _forces(orc, box)
        p = p * ap + F * bp                                     # 3.5
        V = V0 * np.exp(3.0 * eps)
        p_eps += (dt / 2.0) * (alpha * ke2() + float(Wv.sum()) - 3.0 * Pext * V)   # 3.6
        p *= _chain_half(peta, eta, Q, ke2(), 3.0 * n, kT, dt, cfg.temperaturerespa)
        p_eps *= _chain_half(petaP, etaP, QP, p_eps * p_eps / W, 1.0, kT, dt, cfg.pressurerespa)
        r = np.stack([wrap(r[:, a], box[a]) for a in range(3)], 1)
        if (t + 1) % stride == 0 or t == nsteps - 1:
            record(t + 1)
    for a in range(3):
        orc.st.box[a] = float(Lmax[a])
    return recs, dict(r=r, p=p, eta=eta, peta=peta, p_eps=p_eps, eps=eps, etaP=etaP, petaP=petaP, box=box)
