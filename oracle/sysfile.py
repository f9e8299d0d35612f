"""TEST INFRASTRUCTURE: writes an MDSystem + MDConfig as the text system file read by the oracle
harness (oracle/ref/harness.cpp), and runs the harness.  Only tests/ and the golden-fixture
script use this module."""
from __future__ import annotations

import os
import subprocess
import tempfile
from typing import Optional

import numpy as np

from moltwister_gb300.system import MDConfig, MDSystem

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "mtref")


def _f(x: float) -> str:
    return repr(float(x))


def write_sysfile(path: str, s: MDSystem, cfg: MDConfig, with_state: bool = True) -> None:
    lines = ["box " + " ".join(_f(v) for v in s.box)]
    for k in range(s.n):
        lines.append(f"atom {s.ids[k]} {_f(s.r[k,0])} {_f(s.r[k,1])} {_f(s.r[k,2])} "
                     f"{_f(s.q[k])} {_f(s.m[k])} {int(bool(s.mobile[k]))}")
    for t in s.nonbonded:
        lines.append(f"nonbonded {t.id1} {t.id2} {t.kind} " + " ".join(t.command_args()))
    for t in s.bond_terms:
        lines.append(f"bond {t.id1} {t.id2} {t.kind} {t.criterion} {_f(t.crit_r0)} " + " ".join(_f(a) for a in t.args))
    for t in s.angle_terms:
        lines.append(f"angle {t.id1} {t.id2} {t.id3} {t.kind} {t.criterion} {_f(t.crit_r0)} " + " ".join(_f(a) for a in t.args))
    for t in s.dihedral_terms:
        args = [_f(a) for a in t.args]
        if t.kind == "Harm":   # K (double) D N (ints)
            args = [_f(t.args[0]), str(int(t.args[1])), str(int(t.args[2]))]
        lines.append(f"dihedral {t.id1} {t.id2} {t.id3} {t.id4} {t.kind} {t.criterion} {_f(t.crit_r0)} " + " ".join(args))
    for k, v in cfg.reference_cfg_lines():
        lines.append(f"cfg {k} {v}")
    if with_state:
        if s.p is not None:
            for k in range(s.n):
                lines.append(f"mom {_f(s.p[k,0])} {_f(s.p[k,1])} {_f(s.p[k,2])}")
        if s.nhT_eta is not None:
            lines.append("nhT_eta " + " ".join(_f(v) for v in s.nhT_eta))
        if s.nhT_peta is not None:
            lines.append("nhT_peta " + " ".join(_f(v) for v in s.nhT_peta))
        if s.nhP_eta is not None:
            lines.append("nhP_eta " + " ".join(_f(v) for v in s.nhP_eta))
        if s.nhP_peta is not None:
            lines.append("nhP_peta " + " ".join(_f(v) for v in s.nhP_peta))
        if s.p_eps is not None:
            lines.append(f"p_eps {_f(s.p_eps)}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def run_harness(args, s: MDSystem, cfg: MDConfig, timeout: Optional[float] = None) -> str:
    """Run `mtref <cmd> SYS ...`; returns stdout."""
    if not os.path.exists(HARNESS):
        raise RuntimeError("oracle harness not built (make -C oracle/ref)")
    with tempfile.TemporaryDirectory() as td:
        sysf = os.path.join(td, "sys.txt")
        write_sysfile(sysf, s, cfg)
        cmd = [HARNESS, args[0], sysf] + [str(a) for a in args[1:]]
        out = subprocess.run(cmd, check=True, capture_output=True, text=True, timeout=timeout)
        return out.stdout


def harness_static(s: MDSystem, cfg: MDConfig):
    from .mtb import read_mtb
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.mtb")
        run_harness(["static", out], s, cfg)
        return read_mtb(out)


def harness_run(s: MDSystem, cfg: MDConfig, nsteps: int, stride: int):
    from .mtb import read_mtb
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.mtb")
        run_harness(["run", out, nsteps, stride], s, cfg)
        return read_mtb(out)


def harness_init(s: MDSystem, cfg: MDConfig, seed: int):
    """The reference's initial state after srand(seed) (oracle/ref/harness.cpp `init`)."""
    from .mtb import read_mtb
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.mtb")
        run_harness(["init", out, int(seed)], s, cfg)
        return read_mtb(out)
