"""TEST INFRASTRUCTURE: the pair-distance histogram of CCmdPairCorrelation::execute
(Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.cpp:182-215) for one frame, restated in numpy with
the same per-pair arithmetic (C3DVector::distToAcrossPBC, Utilities/3DVector.cpp:44-66).  Only
tests/ use it."""
from __future__ import annotations

import numpy as np


def pair_histogram(r: np.ndarray, ia, ib, box, nbins: int, rmin: float, rmax: float, ignore_below: float = -1.0):
    r = np.asarray(r, np.float64)
    prof = np.zeros(nbins, np.int64)
    span = rmax - rmin
    for i in ia:
        d = np.abs(r[i][None, :] - r[np.asarray(ib)])
        for a in range(3):
            w = box[a]
            d[:, a] = np.where(d[:, a] > w / 2.0, w - d[:, a], d[:, a])
        R = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
        keep = ~(R < ignore_below)
        n = (((R[keep] - rmin) / span) * float(nbins)).astype(np.int64)
        n = n[(n >= 0) & (n < nbins)]
        prof += np.bincount(n, minlength=nbins)[:nbins]
    return prof
