"""Parameter gradients on the GPU (mtg_energy_grad, mtg_loss_grad): against central finite
differences of the library's own energies and losses (h = 1e-4 relative; agreement within 1e-4
relative), and against the FP64 reference adjoint of oracle/adjoint.py on the same trajectory
(within 1e-6 relative: both are FP64, they differ only in summation order)."""
import numpy as np
import pytest

from moltwister_gb300 import grad as G
from moltwister_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_case(precision="fp64"):
    s, cfg = W.water(n_mol=64, L=W.water_box_length(64), seed=21, T=300.0, rc=5.5)
    cfg.precision = precision
    cfg.coulomb = "shifted"
    cfg.coulombcutoff = 5.5
    cfg.listskin = 1.0
    cfg.clipforces = False
    cfg.ljshift = 2
    return s, cfg


def params_of(s):
    return [G.lj_sigma(s, "Ow", "Ow"), G.lj_eps(s, "Ow", "Ow"), G.charge(s, {"Ow": 1.0, "Hw": -0.5}),
            G.bond_k(s, 0), G.angle_theta0(s, 0)]


def engine(s, cfg):
    from moltwister_gb300.engine import Engine
    return Engine(s, cfg)


def loss_of(s, nsteps=20):
    return G.RDFLoss.for_types(s, "Ow", "Ow", nsteps=nsteps, checkpoint_every=7, nbins=100, rmax=5.0, width=0.05)


def perturbed_target(e, params, loss):
    base = e.get_params(params)
    pert = base * np.array([1.02, 0.95, 1.03, 1.0, 1.0])
    e.set_params(params, pert)
    _, _, gbar = e.loss_grad(loss, params, with_grad=False)
    e.set_params(params, base)
    return gbar


def test_energy_grad_matches_finite_differences():
    s, cfg = small_case()
    e = engine(s, cfg)
    params = params_of(s)
    base = e.get_params(params)
    U, g = e.energy_grad(params)
    for k in range(len(params)):
        h = 1e-4 * abs(base[k])
        v = base.copy(); v[k] += h; e.set_params(params, v)
        Up = e.energy_grad([])[0]
        v = base.copy(); v[k] -= h; e.set_params(params, v)
        Um = e.energy_grad([])[0]
        e.set_params(params, base)
        fd = (Up - Um) / (2 * h)
        assert abs(g[k] - fd) <= 1e-4 * max(abs(fd), 1e-6 * abs(U)), (k, g[k], fd)


def test_loss_grad_matches_reference_adjoint():
    from oracle import adjoint as A
    s, cfg = small_case()
    e = engine(s, cfg)
    params = params_of(s)
    loss = loss_of(s)
    loss.target = perturbed_target(e, params, loss)
    L, g, gbar = e.loss_grad(loss, params)
    M = A.water_model(s, rc=5.5, q_dir={"Ow": 1.0, "Hw": -0.5}, lj_force_shift=True)
    ta = s.type_names().index("Ow")
    Lo, go, gbo = A.loss_and_grad(M, s.r, s.p, dt=cfg.timestep / 100.0, nsteps=loss.nsteps, ta=ta, tb=ta,
                                  nbins=loss.nbins, rmax=loss.rmax, width=loss.width, target=loss.target,
                                  names=["sigma", "eps", "q", "bond_k", "angle_theta0"])
    assert abs(L - Lo) <= 1e-6 * Lo, (L, Lo)
    assert np.allclose(gbar, gbo, rtol=1e-8, atol=1e-8)
    assert np.allclose(g, go, rtol=1e-6, atol=1e-12 * np.abs(go).max()), (g, go)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_loss_grad_matches_finite_differences(precision):
    s, cfg = small_case(precision)
    e = engine(s, cfg)
    params = params_of(s)
    loss = loss_of(s)
    loss.target = perturbed_target(e, params, loss)
    base = e.get_params(params)
    L, g, _ = e.loss_grad(loss, params)
    for k in range(len(params)):
        h = 1e-4 * abs(base[k])
        v = base.copy(); v[k] += h; e.set_params(params, v)
        Lp = e.loss_grad(loss, params, with_grad=False)[0]
        v = base.copy(); v[k] -= h; e.set_params(params, v)
        Lm = e.loss_grad(loss, params, with_grad=False)[0]
        e.set_params(params, base)
        fd = (Lp - Lm) / (2 * h)
        tol = 1e-4 if precision == "fp64" else 1e-2
        assert abs(g[k] - fd) <= tol * max(abs(fd), 1e-3 * abs(L)), (k, g[k], fd)


def test_torch_function_returns_the_adjoint_gradient():
    import torch
    s, cfg = small_case()
    e = engine(s, cfg)
    params = params_of(s)
    loss = loss_of(s)
    loss.target = perturbed_target(e, params, loss)
    _, g, _ = e.loss_grad(loss, params)
    theta = torch.tensor(e.get_params(params), dtype=torch.float64, requires_grad=True)
    L = G.TrajectoryLoss.apply(theta, e, params, loss)
    (2.0 * L).backward()
    assert np.allclose(theta.grad.numpy(), 2.0 * g, rtol=1e-12, atol=0.0)
