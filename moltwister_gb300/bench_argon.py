"""LJ argon benchmark: the drop-in reference-precision path and the production modes on one system.

    python -m moltwister_gb300.bench_argon [--ncell 10] [--steps 1000]

System (workloads.argon): 4,000 LJ argon atoms on an FCC lattice (10^3 cells) at reduced density
0.8, sigma 3.405 A, eps 0.996 kJ/mol, cutoff 2.5 sigma, neighbour shell 2 A (5^3 cells), NVT
120 K (Nose-Hoover M = 4, RESPA 4), dt = 2 fs, Maxwell-Boltzmann momenta.  This is the system of
the `argon4000_nvt` parity fixture.

Reported (one JSON line): atom-steps/s of
  - `reference`: the reference-precision path (the reference's 1,000-point tables and summation
    order, cell and neighbour lists rebuilt every step, all-pairs Coulomb with its exact skip of
    zero-charge pairs), the drop-in for `moldyn run`.  Its thermostat reproduces the reference's
    chain arithmetic, which diverges on large systems (a non-finite state ends the timed run,
    and the line says where); `reference_nve` times the same path without the thermostat;
  - `fp64` and `mixed`: the production modes (analytic terms, Verlet list with a 1 A skin);
each timed with CUDA events around the run (chunks of 100 steps), with SM clocks sampled during
every timed region.
"""
from __future__ import annotations

import argparse
import json

from .clocks import ClockSampler


def _timed(e, steps: int, chunk: int = 100):
    """(device ms, steps done): chunks of `chunk` steps until `steps` or a non-finite state."""
    from .engine import MTGError
    ms = 0.0
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        try:
            e.run(k)
        except MTGError as err:
            if err.code != -7:
                raise
            break
        ms += e.stats()["device_ms"]
        done += k
    return ms, done


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ncell", type=int, default=10)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    args = ap.parse_args(argv)

    from moltwister_gb300 import workloads as W
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine, device_name
    build()
    out = {"metric": "atom-steps/s", "workload": f"argon{4 * args.ncell ** 3}_nvt", "device": device_name(0)}
    legs = [("reference", "NVT"), ("reference", "NVE"), ("fp64", "NVT"), ("mixed", "NVT")]
    for prec, ens in legs:
        s, cfg = W.argon(ncell=args.ncell)
        cfg.precision = prec
        cfg.ensemble = ens
        if prec != "reference":
            cfg.listskin = 1.0
        e = Engine(s, cfg)
        e.run(args.warmup)
        with ClockSampler(0) as clk:
            ms, done = _timed(e, args.steps)
        st = e.stats()
        leg = {"value": s.n * done / (ms * 1e-3) if done else None, "steps": done, "ms_per_step": ms / done if done else None,
               "clocks": clk.summary()}
        if done < args.steps:
            # the reference's chain arithmetic (its Suzuki-Yoshida weight, CMt::exp and the p_eta
            # clamp) diverges on large systems; the run stops at the first non-finite step end
            leg["stopped"] = f"non-finite thermostat state within steps {args.warmup + done}-{args.warmup + done + 100}"
        if prec != "reference":
            leg["list_builds"] = st["list_builds"]
        out[prec if ens == "NVT" else prec + "_nve"] = leg
        out["atoms"] = s.n
        e.close()
    out["mixed_over_reference_nve"] = out["mixed"]["value"] / out["reference_nve"]["value"]
    out["config"] = {"rho_star": 0.8, "T_K": 120.0, "dt_fs": 2.0, "cutoff": "2.5 sigma (8.51 A)", "shell_A": 2.0,
                     "ensemble": "NVT Nose-Hoover M=4 RESPA 4", "data": "synthetic (FCC lattice, seeded momenta)"}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
