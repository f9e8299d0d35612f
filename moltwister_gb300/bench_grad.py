"""Differentiable short-trajectory loss on water: gradient throughput and checks.

    python -m moltwister_gb300.bench_grad [--n-mol 500] [--steps 200] [--checkpoint 20] [--reps 5]

System: 500 flexible waters (the benchmark's water model) in a 24.7 A box at 300 K, cutoff 8.0 A
(so that the box holds three reference cells and the minimum image), shifted-force Coulomb, FP64,
relaxed by gradient descent and 500 NVT steps.  Loss: squared deviation of the Gaussian-smeared
O-O pair correlation (0-8 A, 160 bins, width 0.05 A) averaged over 200 velocity-Verlet steps at
dt = 0.5 fs from a target made by the same run with sigma_O +2 %, eps_O -5 %, q_O +3 %.
Gradients with respect to sigma_O, eps_O, q_O (q_H = -q_O/2), the O-H bond constant and the
H-O-H angle, with states stored every 20 steps and recomputation in between.

Reported (one JSON line): grads/s (loss + adjoint gradient evaluations per second, wall clock),
the gradient, central finite differences (h = 1e-4 relative) of each component, their Richardson
extrapolation with h/2 (the differences converge slowly on a 200-step chaotic trajectory), the
relative differences, and the mixed-precision forward's gradient against the FP64 one.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-mol", type=int, default=500)
    ap.add_argument("--box", type=float, default=24.7)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--checkpoint", type=int, default=20)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args(argv)

    from moltwister_gb300 import grad as G
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine, device_name
    build()
    s, cfg = G.water_rdf_case(n_mol=args.n_mol, L=args.box)
    cfg.ensemble = "NVT"
    e = Engine(s, cfg)
    e.optimize(400)
    e.run(500)
    params = [G.lj_sigma(s, "Ow", "Ow"), G.lj_eps(s, "Ow", "Ow"), G.charge(s, {"Ow": 1.0, "Hw": -0.5}),
              G.bond_k(s, 0), G.angle_theta0(s, 0)]
    names = ["sigma_O", "eps_O", "q_O", "k_bond", "theta0"]
    loss = G.RDFLoss.for_types(s, "Ow", "Ow", nsteps=args.steps, checkpoint_every=args.checkpoint)
    base = e.get_params(params)
    e.set_params(params, base * np.array([1.02, 0.95, 1.03, 1.0, 1.0]))
    loss.target = e.loss_grad(loss, params, with_grad=False)[2]
    e.set_params(params, base)
    e.loss_grad(loss, params)                          # warm-up
    from .clocks import ClockSampler
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(args.reps):
            L, g, _ = e.loss_grad(loss, params)
        dt = (time.perf_counter() - t0) / args.reps
    t0 = time.perf_counter()
    for _ in range(args.reps):
        e.loss_grad(loss, params, with_grad=False)
    dt_fwd = (time.perf_counter() - t0) / args.reps
    def central(k, rel_h):
        h = rel_h * abs(base[k])
        v = base.copy(); v[k] += h; e.set_params(params, v)
        Lp = e.loss_grad(loss, params, with_grad=False)[0]
        v = base.copy(); v[k] -= h; e.set_params(params, v)
        Lm = e.loss_grad(loss, params, with_grad=False)[0]
        return (Lp - Lm) / (2 * h)

    fd = np.array([central(k, 1e-4) for k in range(len(params))])
    fd2 = np.array([central(k, 0.5e-4) for k in range(len(params))])
    fd_rich = (4.0 * fd2 - fd) / 3.0          # Richardson extrapolation of the two central differences
    e.set_params(params, base)
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-30)
    rel_rich = np.abs(g - fd_rich) / np.maximum(np.abs(fd_rich), 1e-30)
    # mixed-precision forward, FP64 adjoint
    r, p, th = e.get_state()
    cm = G.water_rdf_case(n_mol=args.n_mol, L=args.box)[1]
    cm.precision = "mixed"
    sm = s.copy()
    sm.r, sm.p = r, p
    em = Engine(sm, cm)
    Lm_, gm, _ = em.loss_grad(loss, params)
    out = {"metric": "grads/s", "value": 1.0 / dt, "unit": "loss+gradient evaluations/s", "device": device_name(0),
           "workload": f"water{3 * args.n_mol}_rdf_loss", "steps": args.steps, "checkpoint_every": args.checkpoint,
           "seconds_per_grad": dt, "seconds_per_loss": dt_fwd, "loss": L, "clocks": clk.summary(),
           "params": dict(zip(names, base.tolist())), "grad": dict(zip(names, g.tolist())),
           "fd": dict(zip(names, fd.tolist())), "rel_diff_vs_fd": dict(zip(names, rel.tolist())),
           "max_rel_diff_vs_fd": float(rel.max()),
           "fd_richardson": dict(zip(names, fd_rich.tolist())),
           "rel_diff_vs_fd_richardson": dict(zip(names, rel_rich.tolist())),
           "max_rel_diff_vs_fd_richardson": float(rel_rich.max()),
           "mixed_forward": {"loss": Lm_, "grad": dict(zip(names, gm.tolist())),
                             "rel_diff_vs_fp64": dict(zip(names, (np.abs(gm - g) / np.abs(g)).tolist()))},
           "config": {"box_A": args.box, "cutoff_A": 8.0, "coulomb": "shifted-force 8 A", "dt_fs": 0.5,
                      "rdf": "O-O, 0-8 A, 160 bins, width 0.05 A", "precision": "fp64 forward and adjoint",
                      "target": "sigma_O +2%, eps_O -5%, q_O +3%", "data": "synthetic (seeded)"}}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
