"""Replica-ensemble benchmark: hundreds of independent systems of uneven size in one batch.

    python -m moltwister_gb300.bench_replicas [--nrep 512] [--steps 2000] [--serial-sample 16]

Ensemble (workloads.replica_spec, seeded): each replica LJ argon (sigma 3.405 A, eps 0.996 kJ/mol,
reduced density 0.8, cutoff 2.5 sigma) or flexible water (1.0 g/cm^3, cutoff 10 A, shifted-force
Coulomb), chosen by seed; sizes uniform in 200-20,000 atoms; temperatures uniform in 80-400 K;
pair cutoffs shortened below half the box for the smallest boxes.  Water replicas are relaxed by
300 gradient-descent steps first.  NVT (Nose-Hoover M=4, RESPA 4), dt = 0.5 fs, mixed precision,
one CUDA graph per 100 steps (output every 100 steps); the force kernel's lanes per atom are
picked by the library's autotuner.

Reported (one JSON line): the batch's atom-steps/s (all replicas, CUDA events around the step
graphs), and the same replicas run one at a time (a seeded sample of --serial-sample replicas,
each timed alone, extrapolated to the whole ensemble by their atom counts).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import time

import numpy as np


def _make(args):
    from moltwister_gb300 import workloads as W
    kind, n, T, seed = args
    return W.make_replica(kind, n, T, seed)


def shared_config():
    from moltwister_gb300.system import MDConfig
    return MDConfig(timestep=0.5, ensemble="NVT", temperature=300.0, temperaturerelax=20.0, cutoffradius=10.0,
                    neighshell=1.0, coulomb="shifted", coulombcutoff=10.0, listskin=1.0, precision="mixed",
                    clipforces=True, optlearningrate=2e-5)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nrep", type=int, default=512)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--serial-sample", type=int, default=16)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--workers", type=int, default=8)
    args = ap.parse_args(argv)

    from moltwister_gb300 import workloads as W
    spec = W.replica_spec(args.nrep, seed=args.seed)
    t0 = time.perf_counter()
    # generation on host cores; spawned workers, started before any GPU use
    with mp.get_context("spawn").Pool(args.workers) as pool:
        made = pool.map(_make, spec, chunksize=4)
    gen_s = time.perf_counter() - t0

    from moltwister_gb300.batch import BatchEngine
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine, device_name
    build()
    cfg = shared_config()
    systems = [m[0] for m in made]
    cutoffs = [m[1] for m in made]
    temps = [x[2] for x in spec]
    t0 = time.perf_counter()
    for k, (kind, n, T, seed) in enumerate(spec):
        if kind == "water":
            c = shared_config()
            c.temperature = T
            c.cutoffradius = c.coulombcutoff = cutoffs[k]
            e = Engine(systems[k], c)
            e.optimize(300)
            systems[k].r, _, _ = e.get_state()
            e.close()
    relax_s = time.perf_counter() - t0

    b = BatchEngine(systems, cfg, temperatures=temps, cutoffs=cutoffs)
    ntot = b.n
    b.run_batch(100, out_stride=100)                 # warm-up: graph capture
    from .clocks import ClockSampler
    ms = 0.0
    done = 0
    recs = []
    with ClockSampler(0) as clk:
        while done < args.steps:
            k = min(100, args.steps - done)
            recs += b.run_batch(k, out_stride=100)
            ms += b.stats()["device_ms"]
            done += k
    st = b.stats()
    rate = ntot * args.steps / (ms * 1e-3)
    last = recs[-1][1]
    T_K = last[:, 0] * W.CONV_T
    finite = bool(np.all(np.isfinite(last)))
    b.close()

    # the same replicas one at a time (seeded sample, extrapolated by atom count)
    rng = np.random.default_rng(args.seed + 7)
    sample = rng.choice(len(systems), size=min(args.serial_sample, len(systems)), replace=False)
    s_ms, s_atoms = 0.0, 0
    for k in sample:
        c = shared_config()
        c.temperature = temps[k]
        c.cutoffradius = c.coulombcutoff = cutoffs[k]
        e = Engine(systems[k], c)
        e.run(100, out_stride=100, copy_coords=False)
        e.run(200, out_stride=100, copy_coords=False)
        s_ms += e.stats()["device_ms"] / 200.0
        s_atoms += systems[k].n
        e.close()
    serial_ms_per_step = s_ms * ntot / s_atoms
    serial_rate = ntot / (serial_ms_per_step * 1e-3)
    out = {"metric": "atom-steps/s", "workload": f"replicas_{args.nrep}", "replicas": args.nrep, "atoms": ntot,
           "device": device_name(0), "value": rate, "steps": args.steps, "ms_per_step": ms / args.steps,
           "serial": {"value": serial_rate, "sample": int(len(sample)), "ms_per_step": serial_ms_per_step},
           "speedup_batch_over_serial": rate / serial_rate, "clocks": clk.summary(),
           "graph_steps": st["graph_steps"], "force_team": st["force_team"], "list_builds": st["list_builds"],
           "final_T_K": {"min": float(T_K.min()), "max": float(T_K.max())}, "finite": finite,
           "config": {"argon": "rho* 0.8, LJ 2.5 sigma", "water": "1.0 g/cm3, 10 A, shifted Coulomb",
                      "sizes": "uniform 200-20,000", "T_K": "uniform 80-400", "dt_fs": 0.5, "precision": "mixed",
                      "prep_s": {"generate": gen_s, "relax_water": relax_s}, "data": "synthetic (seeded)"}}
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
