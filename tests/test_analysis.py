"""Pair-distance histograms on the GPU (mtg_pair_histogram) against the numpy restatement of the
reference command's per-frame loop: integer counts, bit-exact."""
import numpy as np
import pytest

from tests import golden_cases as G


@pytest.mark.gpu
@pytest.mark.parametrize("pair", [("Ow", "Ow"), ("Ow", "Hw")])
def test_pair_histogram_matches_reference_loop(pair):
    from moltwister_gb300.engine import Engine
    from oracle.analysis import pair_histogram
    s, cfg, _ = G.load("water648_nvt")
    cfg.precision = "fp64"
    cfg.coulomb = "cutoff"
    cfg.coulombcutoff = cfg.cutoffradius
    e = Engine(s, cfg)
    names = s.type_names()
    ta, tb = names.index(pair[0]), names.index(pair[1])
    got = e.pair_histogram(ta, tb, 200, 0.0, 9.0)
    ia = [i for i, x in enumerate(s.ids) if x == pair[0]]
    ib = [i for i, x in enumerate(s.ids) if x == pair[1]]
    ref = pair_histogram(s.r, ia, ib, s.box, 200, 0.0, 9.0)
    assert np.array_equal(got, ref)
    got2 = e.pair_histogram(ta, tb, 200, 0.0, 9.0, ignore_below=0.5, profile=got.copy())
    assert np.array_equal(got2 - got, pair_histogram(s.r, ia, ib, s.box, 200, 0.0, 9.0, 0.5))


@pytest.mark.gpu
def test_pair_correlation_of_a_run_is_normalised():
    from moltwister_gb300.analysis import PairCorrelation
    from moltwister_gb300.engine import Engine
    s, cfg, _ = G.load("argon500_nvt")
    cfg.precision = "mixed"
    cfg.coulomb = "cutoff"
    cfg.coulombcutoff = cfg.cutoffradius
    e = Engine(s, cfg)
    pc = PairCorrelation("Ar", "Ar", 100, 0.0, 14.0, ignore_below=0.1)
    for _ in range(5):
        e.run(20)
        pc.add_frame(e)
    r, pair, g = pc.result()
    assert pc.frames == 5
    assert abs(g[r > 10.0].mean() - 1.0) < 0.1          # the liquid's g(r) tends to 1
    assert g[r < 2.5].max() == 0.0                        # no overlaps
