"""NVE energy drift of the Kob-Andersen mixture against arithmetic, cutoff treatment and time step.

    python -m moltwister_gb300.bench_drift [--ncell 32] [--steps 80000] [--cases all]

For each case (precision, LJ cutoff treatment, time step): seeded KA system (workloads.kob_andersen,
ncell = 32 gives 131,072 atoms), 200 gradient-descent steps, Maxwell-Boltzmann momenta at T* = 0.75,
2,000 steps of equilibration, then a window of --steps steps at dt = 0.5 fs (twice as many at
0.25 fs) sampled every 10 fs.  One JSON line per case: the slope of E = U + K in kT per atom per
ns with its standard error from 20 block means (bench_kob_andersen._drift), the residual
fluctuation per atom, and the wall time.

The cases separate the sources of drift: with LJ energies shifted at the cutoff (ljshift = 1, the
force jumps there) velocity Verlet heats the system by an amount proportional to the time step,
in FP64 as in mixed precision; with force-shifted LJ (ljshift = 2, continuous forces) both
precisions conserve energy to the same small drift.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

CASES = [("mixed", 1, 0.5), ("mixed", 2, 0.5), ("mixed", 1, 0.25), ("mixed", 2, 0.25), ("fp64", 1, 0.5), ("fp64", 2, 0.5)]


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ncell", type=int, default=32)
    ap.add_argument("--steps", type=int, default=80000)
    ap.add_argument("--cases", default="all", help="all, mixed or fp64")
    ap.add_argument("--seed", type=int, default=3)
    args = ap.parse_args(argv)

    from moltwister_gb300 import workloads as W
    from moltwister_gb300.bench_kob_andersen import _drift
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine, device_name
    build()
    for prec, shift, dt in CASES:
        if args.cases != "all" and prec != args.cases:
            continue
        s, cfg = W.kob_andersen(ncell=args.ncell, seed=args.seed)
        cfg.precision = prec
        cfg.ljshift = shift
        cfg.timestep = dt
        kT = cfg.temperature / W.CONV_T
        e = Engine(s, cfg)
        e.optimize(200)
        r, _, _ = e.get_state()
        e.set_state(r=r, p=W.maxwell_boltzmann(s.m, cfg.temperature, np.random.default_rng(args.seed + 1)))
        e.run(2000)
        n = int(round(args.steps * 0.5 / dt))
        t0 = time.perf_counter()
        out = e.run(n, out_stride=max(1, int(round(20 * 0.5 / dt))), copy_coords=False)
        drift, se, noise = _drift([(o.step, o.U + o.K) for o in out], s.n, kT, dt)
        print(json.dumps({"workload": f"kob_andersen_{s.n}", "device": device_name(0), "precision": prec,
                          "lj": "force-shifted" if shift == 2 else "energy-shifted", "dt_fs": dt, "steps": n,
                          "window_ps": n * dt * 1e-3, "nve_drift_kT_per_atom_per_ns": drift, "stderr": se,
                          "noise_kT_per_atom": noise, "wall_s": time.perf_counter() - t0}), flush=True)
        e.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
