"""TEST INFRASTRUCTURE: the pair-distance histogram of CCmdPairCorrelation::execute
(Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.cpp:182-215) for one frame, restated in numpy with
the same per-pair arithmetic (C3DVector::distToAcrossPBC, Utilities/3DVector.cpp:44-66).  Only
tests/ use it."""
from __future__ import annotations

import numpy as np


def pair_histogram(r: np.ndarray, ia, ib, box, nbins: int, rmin: float, rmax: float, ignore_below: float = -1.0,
                   use_pbc: bool = True):
    """Counts of one frame; without use_pbc (the command's `ignorepbc`) the plain distance
    |r2 - r1| (C3DVector::norm, Utilities/3DVector.cpp)."""
    r = np.asarray(r, np.float64)
    prof = np.zeros(nbins, np.int64)
    span = rmax - rmin
    for i in ia:
        if use_pbc:
            d = np.abs(r[i][None, :] - r[np.asarray(ib)])
            for a in range(3):
                w = box[a]
                d[:, a] = np.where(d[:, a] > w / 2.0, w - d[:, a], d[:, a])
        else:
            d = r[np.asarray(ib)] - r[i][None, :]
        R = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
        keep = ~(R < ignore_below)
        n = (((R[keep] - rmin) / span) * float(nbins)).astype(np.int64)
        n = n[(n >= 0) & (n < nbins)]
        prof += np.bincount(n, minlength=nbins)[:nbins]
    return prof


def dcd_frame(r: np.ndarray, box, shift: float = 0.0):
    """(positions, PBC widths) of one frame as `calculate paircorrelation` reads it back from a DCD
    file the MD loop wrote: coordinates stored as float32 (Utilities/DCDFile.cpp:702-729), the box
    truncated to integers (MDLoop.cpp:248-258), and the periodic box rebuilt around the centre of
    the frame's bounding box (CDCDFile::getCurrentBoundingBox / getCurrentPBC, DCDFile.cpp:614-666),
    whose width is (c + w/2) - (c - w/2) in FP64."""
    x = (np.asarray(r, np.float64) + shift).astype(np.float32).astype(np.float64)
    w = np.array([float(int(b)) for b in box])
    lo, hi = x.min(axis=0), x.max(axis=0)
    c = (lo + hi) / 2.0
    width = (c + w / 2.0) - (c - w / 2.0)
    return x, width


def read_pair_correlation(path: str):
    """(table [nbins, 5] of Distance, Count, PairCorr, RDF, IdGas.RDF; pbc widths [frames, 3]) from
    the text the command prints (CmdPairCorrelation.cpp:255-270) and the harness's pbc lines."""
    rows, pbc = [], []
    for line in open(path):
        f = line.split()
        if not f:
            continue
        if f[0] == "pbc":
            pbc.append([float(v) for v in f[2:5]])
        elif len(f) == 5:
            try:
                rows.append([float(v) for v in f])
            except ValueError:
                pass
    return np.array(rows), np.array(pbc)
