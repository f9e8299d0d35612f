"""Trajectory writers (host code of libmtgpu.so, no GPU): the DCD bytes equal those the
reference's CDCDFile wrote for the same frames (tests/golden/dcd_water648_nvt.bin), and XYZ frames
follow CMDLoop::appendToXYZFile's printf formats (MDLoop.cpp:229-246)."""
import os

import numpy as np
import pytest

from tests import golden_cases as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def built():
    from moltwister_gb300.build import build
    build()


def test_dcd_bytes_match_the_reference_writer(tmp_path):
    from moltwister_gb300.trajectory import dcd_append
    s, cfg, _ = G.load("water648_nvt")
    out = str(tmp_path / "t.dcd")
    for sh in (0.0, 0.125):
        dcd_append(out, s.r + sh, s.box, 100, 25, 0.5)
    ref = open(os.path.join(GOLDEN, "dcd_water648_nvt.bin"), "rb").read()
    got = open(out, "rb").read()
    assert len(got) == len(ref)
    assert got == ref


def test_xyz_frame_format(tmp_path):
    from moltwister_gb300.trajectory import xyz_append
    r = np.array([[0.5, -1.25, 3.0], [1e-7, 12345.678, -0.0001]])
    ids = ["Ow", "Hw"]
    out = str(tmp_path / "t.xyz")
    xyz_append(out, r, ids, 7)
    want = "2\r\nFrame 7\r\n" + "".join("%-15s% -15g%-15g%-15g\r\n" % (ids[k], *r[k]) for k in range(2))
    assert open(out, "rb").read() == want.encode()
