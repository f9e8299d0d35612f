"""The FP64 reference adjoint (oracle/adjoint.py) against central finite differences of its own
loss: the pair-correlation loss of a short flexible-water trajectory, gradients with respect to
sigma_O, eps_O, q_O (q_H = -q_O/2), the O-H bond constant and the H-O-H angle."""
import numpy as np

from oracle import adjoint as A
from moltwister_gb300 import workloads as W

NAMES = ["sigma", "eps", "q", "bond_k", "angle_theta0"]


def small_case():
    s, cfg = W.water(n_mol=64, L=W.water_box_length(64), seed=21, T=300.0, rc=5.5)
    M = A.water_model(s, rc=5.5, q_dir={"Ow": 1.0, "Hw": -0.5}, lj_force_shift=True)
    return s, M


def test_reference_adjoint_matches_finite_differences():
    s, M = small_case()
    names = s.type_names()
    ta = names.index("Ow")
    args = dict(dt=0.005, nsteps=20, ta=ta, tb=ta, nbins=100, rmax=5.0, width=0.05)
    base = dict(M.theta)
    # target: the same run with perturbed parameters
    M.theta = dict(base, sigma=base["sigma"] * 1.02, eps=base["eps"] * 0.95, q=base["q"] * 1.03)
    _, _, tgt = A.loss_and_grad(M, s.r, s.p, target=np.zeros(100), names=[], adjoint=False, **args)
    M.theta = dict(base)
    L, g, _ = A.loss_and_grad(M, s.r, s.p, target=tgt, names=NAMES, **args)
    assert L > 0
    for k, nm in enumerate(NAMES):
        h = 1e-4 * abs(base[nm])
        M.theta = dict(base, **{nm: base[nm] + h})
        Lp = A.loss_and_grad(M, s.r, s.p, target=tgt, names=[], adjoint=False, **args)[0]
        M.theta = dict(base, **{nm: base[nm] - h})
        Lm = A.loss_and_grad(M, s.r, s.p, target=tgt, names=[], adjoint=False, **args)[0]
        M.theta = dict(base)
        fd = (Lp - Lm) / (2 * h)
        assert abs(g[k] - fd) <= 1e-4 * max(abs(fd), 1e-3 * abs(L)), (nm, g[k], fd)
