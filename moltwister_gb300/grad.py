"""Parameter gradients: energies and short-trajectory pair-correlation losses (mtg_energy_grad,
mtg_loss_grad), and a torch.autograd.Function around them.

Parameters are (kind, index, dq) triples of include/mtgpu.h; the helpers below build them from
atom-type names:

    params = [lj_sigma(s, "Ow", "Ow"), lj_eps(s, "Ow", "Ow"), charge(s, {"Ow": 1.0, "Hw": -0.5}),
              bond_k(s, 0), angle_theta0(s, 0)]
    loss = RDFLoss.for_types(s, "Ow", "Ow", target=g_target, nsteps=200, checkpoint_every=20)
    L, dL, gbar = engine.loss_grad(loss, params)

    theta = torch.tensor(engine.get_params(params), requires_grad=True)
    L = TrajectoryLoss.apply(theta, engine, params, loss)
    L.backward()            # theta.grad = dL/dtheta from the adjoint kernels
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

from .system import MDSystem

P_LJ_EPS, P_LJ_SIGMA, P_CHARGE, P_BOND_K, P_BOND_R0, P_ANGLE_K, P_ANGLE_THETA0 = 1, 2, 3, 4, 5, 6, 7


def _pair_index(s: MDSystem, a: str, b: str) -> int:
    names = s.type_names()
    return names.index(a) * len(names) + names.index(b)


def lj_eps(s: MDSystem, a: str, b: str):
    return (P_LJ_EPS, _pair_index(s, a, b), None)


def lj_sigma(s: MDSystem, a: str, b: str):
    return (P_LJ_SIGMA, _pair_index(s, a, b), None)


def charge(s: MDSystem, per_type: Dict[str, float]):
    """theta such that q_i = theta * per_type[type of i] (types absent from the dict keep q)."""
    dq = np.array([per_type.get(t, 0.0) for t in s.ids], np.float64)
    return (P_CHARGE, 0, dq)


def bond_k(s: MDSystem, bond_type: int):
    return (P_BOND_K, int(bond_type), None)


def bond_r0(s: MDSystem, bond_type: int):
    return (P_BOND_R0, int(bond_type), None)


def angle_k(s: MDSystem, angle_type: int):
    return (P_ANGLE_K, int(angle_type), None)


def angle_theta0(s: MDSystem, angle_type: int):
    return (P_ANGLE_THETA0, int(angle_type), None)


@dataclass
class RDFLoss:
    """mtg_loss_desc: nsteps velocity-Verlet steps, Gaussian-smeared pair correlation of two types
    on nbins bins over [0, rmax] with smearing width `width`, squared deviation from `target`."""
    nsteps: int
    checkpoint_every: int
    type_a: int
    type_b: int
    nbins: int
    rmax: float
    width: float
    target: np.ndarray

    @staticmethod
    def for_types(s: MDSystem, a: str, b: str, target: Optional[np.ndarray] = None, nsteps: int = 200,
                  checkpoint_every: int = 20, nbins: int = 160, rmax: float = 8.0, width: float = 0.05) -> "RDFLoss":
        names = s.type_names()
        tgt = np.zeros(nbins) if target is None else np.asarray(target, np.float64)
        return RDFLoss(nsteps, checkpoint_every, names.index(a), names.index(b), nbins, rmax, width, tgt)


def _torch_function():
    import torch

    class TrajectoryLoss(torch.autograd.Function):
        """L(theta) of an RDFLoss on an Engine; backward returns grad_output * dL/dtheta computed by
        the library's adjoint kernels (the engine's state is left unchanged)."""

        @staticmethod
        def forward(ctx, theta, engine, params, loss):
            engine.set_params(params, theta.detach().cpu().double().numpy())
            L, g, _ = engine.loss_grad(loss, params)
            ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
            return torch.as_tensor(L, dtype=theta.dtype, device=theta.device)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None, None

    return TrajectoryLoss


class _Lazy:
    def __getattr__(self, name):
        return getattr(_torch_function(), name)


TrajectoryLoss = _Lazy()


def water_rdf_case(n_mol: int = 500, L: float = 24.7, seed: int = 4, T: float = 300.0, rc: float = 8.0):
    """The pair-correlation loss case: flexible water (the benchmark's model) with cutoff rc <= 8.2 A
    so the box holds >= 3 reference cells and the minimum image, shifted-force Coulomb and
    force-shifted LJ (a truncated force makes the stepped trajectory discontinuous in the
    parameters wherever a pair crosses the cutoff), FP64."""
    from . import workloads as W
    s, cfg = W.water(n_mol=n_mol, L=L, seed=seed, T=T, rc=rc)
    cfg.precision = "fp64"
    cfg.coulomb = "shifted"
    cfg.coulombcutoff = rc
    cfg.neighshell = 0.2
    cfg.listskin = 1.0
    cfg.clipforces = False
    cfg.ljshift = 2              # force-shifted LJ: continuous forces, so the trajectory is smooth in theta
    cfg.optlearningrate = 2e-5
    return s, cfg
