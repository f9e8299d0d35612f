"""NPT in the production modes (fp64, mixed): the reference's MTK barostat and Nose-Hoover chains
(VelVerlet.cpp:57-71, 124-211, MDLoop.cpp:62-83, NHChain.cpp:54-113) driven by the pair virial,
with the MTK barostat mass, the published Suzuki-Yoshida weights and the exponential itself
(oracle/npt.py states the differences from the reference's arithmetic).

CPU tests pin the oracle: its virial is minus the derivative of the energy under a uniform
scaling of positions and box (which includes every bonded term's virial), and its trajectories
conserve the MTK extended energy to the integrator's O(dt^2).  GPU tests compare the fp64 mode with
the oracle step by step (1e-8, the reference-mode trajectory tolerance), the mixed mode with the
oracle at its force error, and check the extended energy and a state round trip.
"""
import numpy as np
import pytest

CONV_T, CONV_PRESS = 120.272, 16388.2461


def npt_case(name):
    from moltwister_gb300 import workloads as W
    if name == "argon1372":
        # LJ argon compressing from -2,000 atm towards 500 atm: the box shrinks by 3 % in
        # 100 steps, and with a 1.6 A skin the production cell grid goes from 4^3 to 3^3 cells
        s, c = W.argon(ncell=7, seed=11, jitter=0.05)
        c.neighshell = 1.0
        c.listskin = 1.6
        c.ljshift = 2
        c.pressurerelax = 2000.0
        W.make_npt(s, c, 500.0, 21)
    elif name == "argon256":
        s, c = W.argon(ncell=4, seed=11, jitter=0.05)
        c.neighshell = 1.0
        c.listskin = 1.0
        c.ljshift = 2
        c.pressurerelax = 2000.0
        c.timestep = 1.0
        W.make_npt(s, c, 500.0, 21)
    elif name == "water648":
        # flexible water: bonds and angles contribute to the virial
        s, c = W.water(n_mol=216, L=W.water_box_length(216), seed=14, rc=6.0)
        c.coulomb, c.coulombcutoff = "shifted", 6.0
        c.ljshift = 2
        c.listskin = 1.0
        c.pressurerelax = 1000.0
        W.make_npt(s, c, 1.0, 22)
    else:
        raise KeyError(name)
    return s, c


def extended_energy(c, n, rec_U, rec_K, V, th):
    """MTK extended energy of a production-mode NPT state (masses as the library sets them)."""
    kT = c.temperature / CONV_T
    tau, tauP = c.temperaturerelax / 100.0, c.pressurerelax / 100.0
    Q = np.full(len(th.peta), kT * tau * tau)
    Q[0] = 3.0 * n * kT * tau * tau
    QP = kT * tauP * tauP
    W = 3.0 * (n + 1.0) * QP
    Pext = c.pressure / CONV_PRESS
    return (rec_U + rec_K + th.p_eps ** 2 / (2.0 * W) + Pext * V + float((th.peta ** 2 / (2.0 * Q)).sum())
            + 3.0 * n * kT * th.eta[0] + kT * float(np.sum(th.eta[1:]))
            + float((np.asarray(th.petaP) ** 2 / (2.0 * QP)).sum()) + kT * float(np.sum(th.etaP)))


# ------------------------------------------------------------------------------------------------
# the oracle, on the CPU
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["water648", "chains108"])
def test_oracle_virial_is_the_volume_derivative(name):
    """sum over atoms of the per-atom virial = -dU/dlambda at lambda = 1 for r -> lambda r,
    L -> lambda L (central difference), with continuous potentials (force-shifted LJ, shifted
    Coulomb); chains108 has bonds, angles and both dihedral kinds."""
    import ctypes as C
    from moltwister_gb300 import workloads as W
    from oracle.oracle import Oracle, _p, lib
    if name == "water648":
        s, c = npt_case("water648")
    else:
        s, c = W.chains(n_chain=27, L=24.0, seed=15)
        c.coulomb, c.coulombcutoff = "shifted", c.cutoffradius
        c.ljshift = 2
    orc = Oracle(s, c)
    n = s.n
    box0 = np.array(s.box, float)
    r0 = np.array(s.r, float)

    def energy_virial(lam):
        orc.r[...] = r0 * lam
        for a in range(3):
            orc.st.box[a] = float(box0[a] * lam)
        F, U, Wv = np.zeros((n, 3)), np.zeros(n), np.zeros(n)
        lib().orc_forces_fp64_vir(C.byref(orc.st), float(c.cutoffradius), _p(F), _p(U), _p(Wv))
        return U.sum(), Wv.sum()

    _, W0 = energy_virial(1.0)
    h = 1e-6
    Up, _ = energy_virial(1.0 + h)
    Um, _ = energy_virial(1.0 - h)
    dUdl = (Up - Um) / (2.0 * h)
    assert abs(W0 + dUdl) <= 1e-6 * max(1.0, abs(W0)), (W0, -dUdl)


def test_oracle_conserves_the_extended_energy():
    """The oracle's step conserves the MTK extended energy to O(dt^2): halving dt cuts the largest
    excursion about fourfold, and at dt = 1 fs it stays within 0.01 kJ/mol (256 atoms)."""
    from oracle.npt import run_npt
    dev = {}
    for dt in (2.0, 1.0):
        s, c = npt_case("argon256")
        c.timestep = dt
        recs, _ = run_npt(s, c, int(400 * 2 / dt), int(50 * 2 / dt))
        H = np.array([rec[8] for rec in recs])
        dev[dt] = np.abs(H - H[0]).max()
    assert dev[1.0] < 0.01, dev
    assert 2.5 < dev[2.0] / dev[1.0] < 6.0, dev


# ------------------------------------------------------------------------------------------------
# the GPU modes
# ------------------------------------------------------------------------------------------------
def _min_image(d, box):
    return d - box * np.round(d / box)


def _compare(name, prec, tol_r, tol_p, tol_V, tol_P):
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine
    from oracle.npt import run_npt
    build()
    s, c = npt_case(name)
    steps, stride = 100, 25
    recs_o, st_o = run_npt(s, c, steps, stride)
    c.precision = prec
    e = Engine(s, c)
    r_scale = float(np.abs(s.r).max())
    p_scale = float(np.abs(recs_o[0][2]).max())
    P_scale = max(abs(rec[6]) for rec in recs_o)
    for k in range(1, len(recs_o)):
        out = e.run(stride, out_stride=stride - 1)
        r, p, th = e.get_state()
        step, r_o, p_o, U_o, K_o, T_o, P_o, V_o, _ = recs_o[k]
        last = out[-1]
        box = np.asarray(th.box)
        assert np.abs(_min_image(r - r_o, box)).max() <= tol_r * r_scale, (k, np.abs(_min_image(r - r_o, box)).max())
        assert np.abs(p - p_o).max() <= tol_p * p_scale, (k, np.abs(p - p_o).max())
        assert abs(last.V - V_o) <= tol_V * V_o, (k, last.V, V_o)
        assert abs(np.prod(box) - V_o) <= tol_V * V_o
        assert abs(last.P - P_o) <= tol_P * P_scale, (k, last.P, P_o)
        assert abs(last.U - U_o) <= tol_P * max(1.0, abs(U_o)), (k, last.U, U_o)
    e.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["argon1372", "water648"])
def test_npt_fp64_matches_oracle(name):
    _compare(name, "fp64", 1e-8, 1e-8, 1e-9, 1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["argon1372", "water648"])
def test_npt_mixed_matches_oracle(name):
    # FP32 pair arithmetic (relative force error ~1e-6), over 100 steps
    _compare(name, "mixed", 1e-5, 1e-4, 1e-6, 1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_npt_extended_energy(prec):
    """400 steps of 256 argon atoms at dt = 1 fs, read every 50 steps: the extended energy stays
    within 0.02 kJ/mol (the oracle: 0.003)."""
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine
    build()
    s, c = npt_case("argon256")
    c.precision = prec
    e = Engine(s, c)
    H = []
    for k in range(9):
        out = e.run(50 if k else 1, out_stride=49 if k else 1)
        _, _, th = e.get_state()
        last = out[-1]
        H.append(extended_energy(c, s.n, last.U, last.K, last.V, th))
    H = np.array(H)
    assert np.abs(H - H[0]).max() < 0.02, H - H[0]
    e.close()


@pytest.mark.gpu
def test_npt_mixed_state_round_trip():
    """The state (positions, momenta, both chains, p_eps, strain and box) read after 60 steps and
    written back continues within 1e-9 of the straight run."""
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine
    build()
    s, c = npt_case("argon1372")
    c.precision = "mixed"
    e1 = Engine(s, c)
    e1.run(120)
    r1, p1, th1 = e1.get_state()
    e2 = Engine(s, c)
    e2.run(60)
    r, p, th = e2.get_state()
    e3 = Engine(s, c)
    e3.set_state(r=r, p=p, thermo=th)
    e3.run(60)
    r3, p3, th3 = e3.get_state()
    assert np.abs(_min_image(r3 - r1, np.asarray(th1.box))).max() < 1e-9 * np.abs(r1).max()
    assert np.abs(p3 - p1).max() < 1e-9 * np.abs(p1).max()
    assert abs(th3.eps - th1.eps) < 1e-12 and np.allclose(th3.box, th1.box, rtol=1e-12, atol=0)
    for x in (e1, e2, e3):
        x.close()
