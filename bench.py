"""Benchmark: MD atom-steps/s of the GB300 engine on the flexible-water workload.

Workload: 3,000 flexible SPC/E-like waters (9,000 atoms) in a 44.8 A periodic box, NVT 300 K
(Nose-Hoover chain M=4, RESPA 4), dt = 0.5 fs, LJ on O-O (cutoff 10 A), Coulomb within 10 A,
harmonic O-H bonds and H-O-H angles; molecules on a seeded lattice with random orientations,
Maxwell-Boltzmann momenta, relaxed by 400 untimed gradient-descent steps.  Coulomb within 10 A
(`--coulomb`: plain cutoff or shifted force, both new options: the reference has only all-pairs
Coulomb).  Mixed precision (FP32 arithmetic, int64 fixed-point forces).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is device-resident throughput (CUDA events on the engine's stream
around the captured step graphs, L2 flushed between timed chunks of 100 steps); `e2e` is the same
metric through the C ABI with pinned host buffers (state upload, the run, final download), after
one untimed pass of the same calls, by wall clock.  Beside it: the same workload in the FP64 mode
(`fp64`), the mixed-vs-FP64 force error at the final state (`force_error`), and the drop-in
reference-precision GPU path (tables, all-pairs Coulomb, lists every step) on the same atoms
(`reference_mode_gpu`).  The reference arm and `cpu_baseline` time the C restatement of the
reference's MD step (tables, cell and neighbour lists every step, FP64 sums) with this workload's
Coulomb treatment on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from moltwister_gb300.clocks import ClockSampler  # noqa: E402

WORKLOAD = "water9000_nvt"
METRIC = "atom-steps/s"
CHUNK = 100
# DRAM bytes of one force-gather launch on this workload (10 A Coulomb cutoff), from a committed
# ncu capture that names its command
PFORCE_DRAM_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles",
                                "k_pforce_water9000_mixed_dram.json")


def pforce_traffic(coulomb: str):
    """dram__bytes_read.sum + dram__bytes_write.sum per force-gather launch (None when no capture
    of this workload is committed)."""
    if coulomb != "cutoff" or not os.path.exists(PFORCE_DRAM_FILE):
        return None
    with open(PFORCE_DRAM_FILE) as f:
        d = json.load(f)
    return float(d["dram__bytes_read.sum"] + d["dram__bytes_write.sum"])
SIGMA_O, EPS_O = 3.166, 0.650


def make_system(precision: str = "mixed", coulomb: str = "cutoff"):
    from moltwister_gb300 import workloads as W
    s, cfg = W.water(n_mol=3000, L=44.8, seed=2, rc=10.0, dt=0.5)
    cfg.precision = precision
    cfg.coulomb = coulomb
    cfg.coulombcutoff = 10.0
    cfg.listskin = 1.0
    cfg.optlearningrate = 2e-5
    return s, cfg


def shared_config(s, coulomb: str) -> dict:
    """The `config` object both arms print (the physics; precision is the line's `dtype`)."""
    kind = {"shifted": "shifted-force cutoff 10 A", "cutoff": "cutoff 10 A"}[coulomb]
    return {"workload": WORKLOAD, "atoms": int(s.n), "molecules": int(s.n) // 3, "box_A": 44.8, "dt_fs": 0.5,
            "ensemble": "NVT Nose-Hoover M=4 RESPA 4, 300 K", "lj_cutoff_A": 10.0, "coulomb": kind,
            "prep": "seeded lattice, 400 gradient-descent steps (lr 2e-5), untimed"}


# ------------------------------------------------------------------------------------------------
# Algorithmic work (per step): FLOP per unordered pair within cutoff -- 23 for 12-6 LJ, +7 when
# Coulomb is added to an LJ pair, 15 for a Coulomb-only pair -- plus bonds 20 and angles 60.
# ------------------------------------------------------------------------------------------------
def count_pairs(r: np.ndarray, box: np.ndarray, rc: float, is_o: np.ndarray, mol: np.ndarray):
    n = r.shape[0]
    lj_coul = 0
    coul = 0
    for a in range(0, n, 512):
        d = r[a:a + 512, None, :] - r[None, :, :]
        d -= box * np.rint(d / box)
        r2 = (d * d).sum(-1)
        idx = np.arange(a, min(a + 512, n))
        upper = np.arange(n)[None, :] > idx[:, None]
        intra = mol[idx][:, None] == mol[None, :]
        within = (r2 < rc * rc) & upper & ~intra
        oo = is_o[idx][:, None] & is_o[None, :]
        lj_coul += int((within & oo).sum())
        coul += int((within & ~oo).sum())
    return lj_coul, coul


def algorithmic_flops(s, r, cfg) -> float:
    is_o = np.array([i == "Ow" for i in s.ids])
    ljc, c = count_pairs(r, s.box, cfg.cutoffradius, is_o, s.mol_index())
    return 30.0 * ljc + 15.0 * c + 20.0 * len(s.bonds) + 60.0 * len(s.angles)


def reduce_over_ranks(ms: float, atom_steps: float, device=None):
    """(largest timed-region ms over ranks, atom-steps of all ranks); the local values when no
    process group is initialised.  Replicas only: no data crosses ranks but these two scalars."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return ms, atom_steps
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    a = torch.tensor([atom_steps], dtype=torch.float64, device=device)
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    return float(t.item()), float(a.item())


_FLUSH = None


def flush_l2():
    """Write 256 MiB (twice the 129 MB L2) on the current device."""
    global _FLUSH
    import torch
    if _FLUSH is None:
        _FLUSH = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    _FLUSH.fill_(1.0)
    torch.cuda.synchronize()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference step (tables, cell and neighbour lists
# every step, FP64 sums), threaded over atoms on every host core
# ------------------------------------------------------------------------------------------------
def cpu_baseline(s, cfg, coulomb: str, budget_s: float = 20.0, max_steps: int = 20):
    from oracle import oracle as O
    from moltwister_gb300.system import MDConfig
    c = MDConfig(**{k: getattr(cfg, k) for k in cfg.__dataclass_fields__})
    c.precision = "reference"
    c.coulomb = coulomb
    orc = O.Oracle(s, c)
    t0 = time.perf_counter()
    orc.run_ref(1, 1)             # one step, to size the sample
    one = time.perf_counter() - t0
    steps = int(max(1, min(max_steps, budget_s // max(one, 1e-9))))
    t0 = time.perf_counter()
    orc.run_ref(steps, steps)
    dt = time.perf_counter() - t0
    return {"value": s.n * steps / dt, "unit": METRIC, "cores": host_threads(), "kind": "port",
            "sample": f"{steps} MD steps of the 9,000-atom water system (its lattice start: the cost of a step "
                      f"does not depend on the relaxation) after 1 untimed step, reference "
                      f"arithmetic (1000-point tables, cell + neighbour lists every step, FP64 sums) with "
                      f"Coulomb {coulomb} at 10 A over the neighbour list (the reference's only Coulomb is "
                      f"all-pairs), atoms split over {host_threads()} threads",
            "seconds": dt}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    s, cfg = make_system("mixed", args.coulomb)
    base = cpu_baseline(s, cfg, args.coulomb, budget_s=min(60.0, 10.0 * max(1, args.steps)),
                        max_steps=max(1, min(args.steps, 20)))
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "impl": "reference", "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": shared_config(s, args.coulomb),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------------
# Our arm
# ------------------------------------------------------------------------------------------------
def timed_device(e, steps: int, chunk: int = CHUNK):
    """Device ms of exactly `steps` steps, run in chunks with an L2 flush between chunks."""
    total = 0.0
    done = 0
    builds = 0
    launches = 0
    while done < steps:
        n = min(chunk, steps - done)
        e.run(n, out_stride=chunk, copy_coords=False)   # one output step (energies, record) per chunk
        st = e.stats()
        total += st["device_ms"]
        builds += st["list_builds"]
        launches += st["kernel_launches"]
        done += n
        flush_l2()
    return total, builds, launches


def pinned(n):
    import torch
    return torch.empty((n, 3), dtype=torch.float64).pin_memory().numpy()


def e2e_once(e, r_in, p_in, th, steps, r_out, p_out):
    e.set_state(r=r_in, p=p_in, thermo=th)
    recs = e.run(steps, out_stride=CHUNK)
    e.get_state(out=(r_out, p_out))
    return recs


def our_arm(args):
    import torch
    from moltwister_gb300.build import build
    from moltwister_gb300.engine import Engine, device_name
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build()
    s, cfg = make_system("mixed", args.coulomb)
    n = s.n
    e = Engine(s, cfg, device=local)
    # untimed preparation: relax the lattice start by gradient descent (the reference's
    # `moldyn optimizeenergy`), as the Nose-Hoover chain cannot absorb the start's energy release
    e.optimize(400)
    r_relaxed, p_relaxed, th_relaxed = e.get_state()
    # warm-up: graph capture and first list builds
    for _ in range(max(args.warmup, 3)):
        e.run(CHUNK)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    with ClockSampler(local) as clk:
        ms, builds, launches = timed_device(e, args.steps)
    torch.cuda.synchronize()
    ms, atom_steps = reduce_over_ranks(ms, float(n * args.steps), device="cuda")
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    value = atom_steps / (ms / 1e3)

    # per-phase device time (same stream, CUDA events) for the roofline
    phases = e.profile_phases(200)
    # e2e through the C ABI with pinned host buffers: upload r and p, run, download r and p; one
    # untimed pass of the same calls first (graph capture for these chunk lengths)
    r_in, p_in, r_out, p_out = pinned(n), pinned(n), pinned(n), pinned(n)
    r0, p0, th0 = e.get_state()
    r_in[:], p_in[:] = r0, p0
    e2e_once(e, r_in, p_in, th0, args.steps, r_out, p_out)
    t0 = time.perf_counter()
    recs = e2e_once(e, r_in, p_in, th0, args.steps, r_out, p_out)
    e2e_s = time.perf_counter() - t0
    e2e_val = world * n * args.steps / e2e_s
    h2d = 2 * 3 * 8 * n
    d2h = (len(recs) + 1) * 2 * 3 * 8 * n
    r_fin, p_fin = r_out.copy(), p_out.copy()

    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp32+int64", "data": "synthetic",
           "config": shared_config(s, args.coulomb),
           "precision": "mixed: FP32 pair and bonded arithmetic, int64 fixed-point force sums, double-float "
                        "(FP32 hi+lo) positions, momenta and Nose-Hoover chain, FP64 block and system sums",
           "list_skin_A": cfg.listskin,
           "l2": f"flushed (256 MiB write) between timed chunks of {CHUNK} steps",
           "parallelism": "replicas only" if world > 1 else "single GPU",
           "device": device_name(local),
           "e2e": {"value": e2e_val, "unit": METRIC, "h2d_bytes_per_step": h2d / args.steps,
                   "d2h_bytes_per_step": d2h / args.steps, "seconds": e2e_s,
                   "path": "Engine.set_state / run / get_state (C ABI), pinned host buffers, after one untimed pass; "
                           "one run of all steps with no L2 flush (the device-timed value flushes L2 before every "
                           f"chunk of {CHUNK} steps)"},
           "gpu_launches": int(launches),
           "graph_form": e.stats()["graph_form"],
           "list_builds": int(builds),
           "phase_ms": phases}
    if rank == 0:
        pk, kind = peaks()
        clk_s = clk.summary()
        # the same workload in FP64 and the mixed-vs-FP64 force error at the final state
        s64, c64 = make_system("fp64", args.coulomb)
        s64.r = r_relaxed
        s64.p = p_relaxed
        e64 = Engine(s64, c64, device=local)
        for _ in range(max(args.warmup, 3)):
            e64.run(CHUNK)
        ms64, _, _ = timed_device(e64, args.steps)
        e64.set_state(r=r_fin, p=p_fin)
        F64, U64 = e64.forces()
        e.set_state(r=r_fin, p=p_fin)
        Fm, Um = e.forces()
        rms = float(np.sqrt(((Fm - F64) ** 2).sum() / (F64 ** 2).sum()))
        mx = float(np.abs(Fm - F64).max() / np.abs(F64).max())
        out["fp64"] = {"value": n * args.steps / (ms64 / 1e3), "unit": METRIC, "ms_per_step": ms64 / args.steps,
                       "mixed_over_fp64": (ms64 / ms)}
        out["force_error"] = {"rel_rms": rms, "max_over_max_force": mx, "energy_rel": float(abs(Um.sum() - U64.sum()) / abs(U64.sum())),
                              "against": "this library's FP64 mode at the final state of the timed run (the FP64 "
                                         "mode matches the FP64 oracle to 1e-10 in the parity tests)"}
        e64.close()
        # the drop-in path on the same atoms: reference precision, tables, all-pairs Coulomb,
        # cell and neighbour lists every step
        sr, cr = make_system("reference", "allpairs")
        sr.r = r_fin
        sr.p = p_fin
        er = Engine(sr, cr, device=local)
        er.run(2)
        nref = max(2, min(args.steps, 10))
        msr, _, _ = timed_device(er, nref, chunk=nref)
        out["reference_mode_gpu"] = {"value": n * nref / (msr / 1e3), "unit": METRIC, "steps": nref,
                                     "ms_per_step": msr / nref,
                                     "path": "reference precision (the reference's tables and summation order, "
                                             "all-pairs Coulomb, lists every step), same 9,000 atoms"}
        er.close()
        # roofline of the force gather: FP32 pipe (no tensor-core work on this path)
        props = torch.cuda.get_device_properties(local)
        sm_max = pk.get("sm_max_mhz", 2070.0)
        fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
        flops = algorithmic_flops(s, r_fin, cfg)
        fms = phases["force"]
        achieved = flops / (fms * 1e-3) / 1e12
        out["roofline"] = {"bound": "fp32", "kernel": "k_pforce (force gather)", "achieved": achieved,
                           "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                           "peak_source": f"FP32 SIMT peak {props.multi_processor_count} SM x 128 lanes x 2 x "
                                          f"{sm_max:.0f} MHz (sm_max_mhz {kind} in MEASURED_PEAKS.json)",
                           "algorithmic_flop_per_launch": flops, "launch_ms": fms,
                           "traffic": pforce_traffic(args.coulomb),
                           "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one k_pforce launch "
                                           "(step loop, no energy) of this workload, from a committed ncu "
                                           "capture (not measured in this run): the Verlet list read once"}
        # integrator: HBM-bound per-atom kernels (kick-drift and second kick, without the step end)
        kd = phases["kick_drift"] + phases["kick_reduce"]
        out["roofline_integrator"] = {"bound": "hbm", "kernels": "k_mkick_drift + k_mkick2",
                                      "achieved": 148.0 * n / (kd * 1e-3) / 1e9,
                                      "peak": pk["hbm_gbs"], "unit": "GB/s",
                                      "frac": 148.0 * n / (kd * 1e-3) / 1e9 / pk["hbm_gbs"],
                                      "peak_source": kind}
        out["clocks"] = clk_s
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(s, cfg, args.coulomb)
        print(json.dumps(out))
    e.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--coulomb", default="cutoff", choices=["cutoff", "shifted"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return our_arm(args)


if __name__ == "__main__":
    sys.exit(main())
