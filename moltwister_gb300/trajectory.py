"""Trajectory output of `moldyn run` (DCD and XYZ files at every output step, MDLoop.cpp:390-397)
through the library's writers, which reproduce the reference's byte layout."""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from .engine import MTG_OK, MTGError, OutputRecord, _ptr, load_library


def dcd_append(path: str, r: np.ndarray, box, num_steps: int, out_stride: int, timestep_fs: float) -> None:
    lib = load_library()
    rr = np.ascontiguousarray(r, np.float64)
    b = np.ascontiguousarray(box, np.float64)
    rc = lib.mtg_dcd_append(path.encode(), int(rr.shape[0]), _ptr(rr), _ptr(b), int(num_steps), int(out_stride),
                            float(timestep_fs))
    if rc != MTG_OK:
        raise MTGError(rc, f"cannot write {path}")


def xyz_append(path: str, r: np.ndarray, ids: List[str], step: int) -> None:
    lib = load_library()
    rr = np.ascontiguousarray(r, np.float64)
    names = (C.c_char_p * len(ids))(*[x.encode() for x in ids])
    rc = lib.mtg_xyz_append(path.encode(), int(rr.shape[0]), _ptr(rr), C.cast(names, C.c_void_p), int(step))
    if rc != MTG_OK:
        raise MTGError(rc, f"cannot write {path}")


class TrajectoryWriter:
    """Output-step callback for Engine.run: appends the frame to a DCD and/or an XYZ file as the
    reference does (`moldyn cfg` outdcdfile / outxyzfile).  The DCD box is the current box (under
    NPT scaled from the output volume)."""

    def __init__(self, engine, num_steps: int, out_stride: int, dcd: Optional[str] = None, xyz: Optional[str] = None):
        self.engine, self.num_steps, self.out_stride = engine, num_steps, out_stride
        self.dcd, self.xyz = dcd, xyz
        s = engine.system
        self.ids = list(s.ids)
        self.box0 = np.asarray(s.box, np.float64)
        self.dt = engine.config.timestep

    def __call__(self, rec: OutputRecord) -> bool:
        if rec.r is None:
            raise ValueError("run with copy_coords=True to write trajectories")
        box = self.box0 * (rec.V / float(np.prod(self.box0))) ** (1.0 / 3.0)
        if self.dcd:
            dcd_append(self.dcd, rec.r, box, self.num_steps, self.out_stride, self.dt)
        if self.xyz:
            xyz_append(self.xyz, rec.r, self.ids, rec.step)
        return False
