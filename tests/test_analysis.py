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


# --- the reference's own `calculate paircorrelation` (tests/golden/paircorr_water648_nvt.npz) ---

def _paircorr_cases():
    import json
    import os
    d = np.load(os.path.join(G.GOLDEN, "paircorr_water648_nvt.npz"))
    keys = sorted({k.split("__")[0] for k in d.files if "__" in k})
    return d, keys, {k: json.loads(str(d[k + "__args"])) for k in keys}


def _parse_args(args):
    id1, id2, nbins, rmin, rmax = args[0], args[1], int(args[2]), float(args[3]), float(args[4])
    ignore = float(args[args.index("ignoredistbelow") + 1]) if "ignoredistbelow" in args else -1.0
    return id1, id2, nbins, rmin, rmax, ignore, "ignorepbc" not in args


@pytest.mark.parametrize("key", ["Ow_Hw", "Ow_Ow_ignore", "Hw_Hw_nopbc"])
def test_oracle_pair_histogram_matches_the_reference_command(key):
    """The numpy restatement of the command's per-frame loop, fed the frames as the command reads
    them back from the DCD file (float32 coordinates, integer box, PBC around the bounding-box
    centre), gives the command's own counts bit for bit, and its PBC widths are the command's."""
    from oracle.analysis import dcd_frame, pair_histogram
    d, _, args = _paircorr_cases()
    s, _, _ = G.load("water648_nvt")
    id1, id2, nbins, rmin, rmax, ignore, pbc = _parse_args(args[key])
    ia = [i for i, x in enumerate(s.ids) if x == id1]
    ib = [i for i, x in enumerate(s.ids) if x == id2]
    total = np.zeros(nbins, np.int64)
    for f in range(int(d["nframes"])):
        x, w = dcd_frame(s.r, s.box, f * float(d["shift"]))
        assert np.array_equal(w, d[key + "__pbc"][f])
        total += pair_histogram(x, ia, ib, w, nbins, rmin, rmax, ignore, use_pbc=pbc)
    assert np.array_equal(total, d[key + "__table"][:, 1].astype(np.int64))


@pytest.mark.gpu
@pytest.mark.parametrize("key", ["Ow_Hw", "Ow_Ow_ignore"])
def test_gpu_pair_correlation_matches_the_reference_command(key):
    """mtg_pair_histogram on the frames the command reads, then the command's normalisation:
    counts bit for bit, PairCorr and RDF to the 6 decimals the command prints."""
    from moltwister_gb300.analysis import PairCorrelation
    from moltwister_gb300.engine import Engine
    from oracle.analysis import dcd_frame
    d, _, args = _paircorr_cases()
    s, cfg, _ = G.load("water648_nvt")
    cfg.precision, cfg.coulomb, cfg.coulombcutoff = "fp64", "cutoff", cfg.cutoffradius
    id1, id2, nbins, rmin, rmax, ignore, _ = _parse_args(args[key])
    pc = PairCorrelation(id1, id2, nbins, rmin, rmax, ignore_below=ignore)
    for f in range(int(d["nframes"])):
        x, w = dcd_frame(s.r, s.box, f * float(d["shift"]))
        sf = s.copy()
        sf.r, sf.box = x, w          # as read back: unwrapped, so every distance is the command's
        e = Engine(sf, cfg)
        pc.add_frame(e)
        e.close()
    table = d[key + "__table"]
    assert np.array_equal(pc.profile, table[:, 1].astype(np.int64))
    r, pair, rdf = pc.result()
    assert np.allclose(r, table[:, 0], atol=5e-5)
    assert np.allclose(pair, table[:, 2], atol=5e-7)
    assert np.allclose(rdf, table[:, 3], atol=5e-7 * np.maximum(1.0, np.abs(table[:, 3])))
