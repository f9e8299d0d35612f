"""Analysis on the GPU: the pair correlation of `calculate paircorrelation`
(Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.cpp:78-260) accumulated over frames of a run."""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class PairCorrelation:
    """Ordered-pair distance histogram of atom IDs id1, id2 over frames (mtg_pair_histogram), and
    the command's normalisation: pairCorr = profile / (N1 frames), ideal-gas pair count
    4 pi r^2 dr <N2 / V>, rdf = pairCorr / idGasPairCorr, r at the bin centres."""
    id1: str
    id2: str
    nbins: int
    rmin: float
    rmax: float
    ignore_below: float = -1.0
    profile: np.ndarray = field(init=False)
    frames: int = field(init=False, default=0)
    n1: int = field(init=False, default=0)
    sum_n2_over_v: float = field(init=False, default=0.0)

    def __post_init__(self):
        self.profile = np.zeros(self.nbins, np.int64)

    def add_frame(self, engine) -> None:
        """Counts the engine's current positions as one frame."""
        s = engine.system
        names = s.type_names()
        engine.pair_histogram(names.index(self.id1), names.index(self.id2), self.nbins, self.rmin, self.rmax,
                              self.ignore_below, self.profile)
        box = np.asarray(engine.get_state()[2].box)
        if not np.all(box > 0):
            box = np.asarray(s.box)
        self.n1 = sum(1 for x in s.ids if x == self.id1)
        n2 = sum(1 for x in s.ids if x == self.id2)
        self.sum_n2_over_v += n2 / float(np.prod(box))
        self.frames += 1

    def result(self):
        """(r, pair correlation [#], rdf) as the command computes them (CmdPairCorrelation.cpp:236-246)."""
        dr = (self.rmax - self.rmin) / self.nbins
        r = 0.5 * (2 * np.arange(self.nbins) + 1) * dr + self.rmin
        ideal = 4.0 * np.pi * r * r * dr * (self.sum_n2_over_v / self.frames)
        pair = self.profile / (self.n1 * self.frames)
        return r, pair, pair / ideal
