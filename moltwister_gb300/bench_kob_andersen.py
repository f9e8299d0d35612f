"""Kob-Andersen benchmark: mixed precision vs plain FP64 on the same GPU, force error and NVE drift.

    python -m moltwister_gb300.bench_kob_andersen [--ncell 64] [--steps 20000] [--fp64-steps 1000]

System: the Kob-Andersen 80:20 binary LJ mixture at reduced density 1.2 (workloads.kob_andersen;
ncell = 64 gives 1,048,576 atoms), cutoff 2.5 sigma_ab per pair with energies shifted to zero at
the cutoffs, LJ reduced units mapped to sigma = 1 A, eps = 1 kJ/mol, m = 1 g/mol (T* = 0.75 is
90.2 K, dt* = 0.005 is 0.5 fs).  Atoms placed uniformly at random (seeded; --placement lattice:
jittered FCC sites) with a random A/B assignment, relaxed by gradient descent in stages of growing
learning rate (workloads.relax_random) and --relax more steps, then Maxwell-Boltzmann momenta at T*.

Reported (one JSON line):
  - atom-steps/s of the mixed and the FP64 path (CUDA events around the step graphs), and their ratio;
  - force error of the mixed path against the FP64 path on the same positions (the configuration
    at the end of the mixed run): relative RMS |F_mixed - F_fp64| / |F_fp64| and the largest
    component error relative to the largest force (the FP64 GPU path is itself checked against
    the FP64 CPU oracle at small sizes by the tests).  Pairs within rounding of a cutoff can be
    counted by one precision and not the other; the truncated force there (0.04 eps/sigma for AA)
    then shows in the maximum, not in the RMS;
  - NVE energy drift: slope of a linear fit of E = U + K, in kT per atom per ns, with its
    standard error from the fit of block means (20 contiguous blocks, so that the correlated
    velocity-Verlet energy fluctuation enters as noise).  The mixed path's drift comes from a
    separate run of --drift-steps steps continuing the timed run, sampled every --drift-stride
    steps: the fitted slope of a 10 ps window scatters by about 1e-3 kT per atom per ns between
    trajectories at 10^6 atoms, too much to resolve the 1e-4 target.  The FP64 run (shorter) is
    reported the same way.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def _drift(recs, n, kT, dt_fs, nblock=20):
    """(slope, standard error, residual std) of E = U + K against time, in kT per atom (per ns)."""
    t_ns = np.array([st for st, _ in recs], float) * dt_fs * 1e-6
    E = np.array([en for _, en in recs]) / (n * kT)
    if len(E) < 3:
        return None, None, None
    fit = np.polyfit(t_ns, E, 1)
    noise = float(np.std(E - np.polyval(fit, t_ns)))
    se = None
    if len(E) >= 4 * nblock:
        m = len(E) // nblock * nblock
        tb = t_ns[:m].reshape(nblock, -1).mean(1)
        Eb = E[:m].reshape(nblock, -1).mean(1)
        fb = np.polyfit(tb, Eb, 1)
        res = Eb - np.polyval(fb, tb)
        se = float(np.sqrt((res ** 2).sum() / (nblock - 2) / ((tb - tb.mean()) ** 2).sum()))
    return float(fit[0]), se, noise


def _timed_run(e, steps, chunk=100):
    ms = 0.0
    done = 0
    recs = []
    while done < steps:
        k = min(chunk, steps - done)
        out = e.run(k, out_stride=k, copy_coords=False)
        ms += e.stats()["device_ms"]
        done += k
        if out:
            recs.append((done, out[-1].U + out[-1].K))   # (global step, total energy)
    return ms, recs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ncell", type=int, default=64)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--fp64-steps", type=int, default=1000)
    ap.add_argument("--relax", type=int, default=200)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--drift-steps", type=int, default=80000)
    ap.add_argument("--drift-stride", type=int, default=20)
    ap.add_argument("--placement", choices=("random", "lattice"), default="random")
    args = ap.parse_args(argv)

    from moltwister_gb300 import workloads as W
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine, device_name
    build()
    s, cfg = W.kob_andersen(ncell=args.ncell, seed=args.seed, placement=args.placement)
    n = s.n
    kT = cfg.temperature / W.CONV_T
    t0 = time.perf_counter()
    if args.placement == "random":
        s.r = W.relax_random(s, cfg)
    em = Engine(s, cfg)
    em.optimize(args.relax)
    r, _, _ = em.get_state()
    rng = np.random.default_rng(args.seed + 1)
    p = W.maxwell_boltzmann(s.m, cfg.temperature, rng)
    em.set_state(r=r, p=p)
    setup_s = time.perf_counter() - t0

    # mixed: throughput and NVE drift from the relaxed start
    from .clocks import ClockSampler
    em.run(100)                                 # warm-up: graph capture, autotuner
    with ClockSampler(0) as clk_m:
        ms_m, recs_m = _timed_run(em, args.steps)

    # FP64 on the same final state: force error on that (equilibrated) configuration, then its
    # own throughput and drift over a shorter run from there
    r, p, _ = em.get_state()
    c64 = W.MDConfig(**{k: getattr(cfg, k) for k in cfg.__dataclass_fields__})
    c64.precision = "fp64"
    s64 = s.copy()
    s64.r = r
    s64.p = p
    e64 = Engine(s64, c64)
    Fm, _ = em.forces()
    F64, _ = e64.forces()
    dF = Fm - F64
    rms = float(np.sqrt((dF ** 2).sum() / (F64 ** 2).sum()))
    mx = float(np.abs(dF).max() / np.abs(F64).max())
    rms_atom = float(np.sqrt((dF ** 2).sum(1).mean()))
    e64.run(20)
    with ClockSampler(0) as clk_64:
        ms_64, recs_64 = _timed_run(e64, args.fp64_steps)
    rate_m = n * args.steps / (ms_m * 1e-3)
    rate_64 = n * args.fp64_steps / (ms_64 * 1e-3)
    builds_m = em.stats()["list_builds"]
    drift_t, se_t, _ = _drift(recs_m, n, kT, cfg.timestep)
    # mixed NVE drift over a long window continuing the timed run
    recs_d = []
    if args.drift_steps > 0:
        out_d = em.run(args.drift_steps, out_stride=args.drift_stride, copy_coords=False)
        recs_d = [(args.steps + o.step, o.U + o.K) for o in out_d]
    drift_m, se_m, noise_m = _drift(recs_d, n, kT, cfg.timestep)
    drift_64, se_64, noise_64 = _drift(recs_64, n, kT, cfg.timestep)
    out = {
        "metric": "atom-steps/s", "workload": f"kob_andersen_{n}", "atoms": n, "device": device_name(0),
        "mixed": {"value": rate_m, "steps": args.steps, "ms_per_step": ms_m / args.steps, "list_builds": builds_m,
                  "force_team": em.stats()["force_team"], "graph_form": em.stats()["graph_form"],
                  "nve_drift_kT_per_atom_per_ns": drift_m, "nve_drift_stderr": se_m,
                  "nve_noise_kT_per_atom": noise_m, "nve_drift_window_steps": args.drift_steps,
                  "nve_drift_stride": args.drift_stride,
                  "timed_run_drift": {"value": drift_t, "stderr": se_t, "window_steps": args.steps}},
        "fp64": {"value": rate_64, "steps": args.fp64_steps, "ms_per_step": ms_64 / args.fp64_steps,
                 "nve_drift_kT_per_atom_per_ns": drift_64, "nve_drift_stderr": se_64, "nve_noise_kT_per_atom": noise_64},
        "speedup_mixed_over_fp64": rate_m / rate_64,
        "clocks": {"mixed": clk_m.summary(), "fp64": clk_64.summary()},
        "force_error_mixed_vs_fp64": {"rel_rms": rms, "max_rel_to_max_force": mx, "rms_abs_kJ_mol_A": rms_atom,
                                      "configuration": f"after the {args.steps}-step mixed NVE run"},
        "config": {"rho_star": 1.2, "T_star": 0.75, "dt_fs": cfg.timestep, "cutoff": "2.5 sigma_ab per pair, shifted",
                   "skin_A": cfg.listskin,
                   "relax": (f"{sum(k for _, k in W.RANDOM_RELAX_STAGES)} staged gradient-descent steps (learning rates "
                             f"{', '.join(str(lr) for lr, _ in W.RANDOM_RELAX_STAGES)}) + " if args.placement == "random" else "")
                            + f"{args.relax} gradient-descent steps", "setup_s": setup_s,
                   "data": ("synthetic (seeded uniform random placement, random A/B)" if args.placement == "random"
                            else "synthetic (seeded FCC sites, random A/B, jitter 0.05)")},
    }
    print(json.dumps(out))
    em.close()
    e64.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
