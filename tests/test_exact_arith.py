"""The exact-arithmetic steps of the reference-precision all-pairs Coulomb kernel, restated in C
(tests/exact_arith/exact_arith.c), against the FP64 operations they replace: the float distance
(float)sqrt(x*x + y*y + z*z), the FP64 quotient of two floats, and the minimum-image test
|c - v| > w/2, on seeded random inputs and on inputs at and next to their rounding boundaries.
Bit-identical on every input; the kernel itself is checked bit for bit against the oracle on the
GPU (test_gpu_parity.py::test_reference_coulomb_bit_exact)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exact_arith_bit_identical(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "exact_arith")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "exact_arith", "exact_arith.c"), "-lm"],
                   check=True)
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "R mismatches 0" in r.stdout and "q mismatches 0" in r.stdout and "image mismatches 0" in r.stdout
