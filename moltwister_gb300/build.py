"""Builds libmtgpu.so (the CUDA engine behind include/mtgpu.h) in-tree, for sm_103a only.

    python -m moltwister_gb300.build

Each translation unit is compiled by nvcc in parallel into moltwister_gb300/_build/, then linked
into moltwister_gb300/_build/libmtgpu.so with the CUDA runtime linked statically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmtgpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE]

# (source, extra flags).  The reference-mode kernels are compiled without fused multiply-adds so
# their FP64 arithmetic rounds like the reference's; the table generator likewise on the host.
UNITS = [
    ("ref_kernels.cu", ["-fmad=false"]),
    ("md_kernels.cu", ["-Xptxas", "-v"] if os.environ.get("MTG_PTXAS_VERBOSE") else []),
    ("api.cu", ["-Xcompiler", "-ffp-contract=off"]),
    ("adjoint.cu", []),
    ("tables.cpp", ["-Xcompiler", "-ffp-contract=off"]),
    ("writers.cpp", []),
    ("init_state.cpp", ["-Xcompiler", "-ffp-contract=off"]),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "mtgpu.h"))
    jobs = []
    objs = []
    for src, extra in UNITS:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
