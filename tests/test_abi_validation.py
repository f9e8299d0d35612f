"""Input validation of mtg_create (no GPU needed: every check runs before any device work).  The
reference prints and carries on; the C ABI returns a negative MTG_E_* code with a message, and the
binding raises MTGError with that code."""
import numpy as np
import pytest

from moltwister_gb300 import engine as E
from moltwister_gb300 import workloads as W

INVALID, UNSUPPORTED, NONFINITE = -1, -6, -7


@pytest.fixture(scope="module", autouse=True)
def built():
    from moltwister_gb300.build import build
    build()


def create_code(s, c):
    with pytest.raises(E.MTGError) as ei:
        E.Engine(s, c)
    return ei.value.code, str(ei.value)


def test_bad_lj_shift():
    s, c = W.argon(ncell=2)
    c.precision = "mixed"
    c.ljshift = 3
    code, msg = create_code(s, c)
    assert code == INVALID and "lj_shift" in msg


def test_npt_in_the_production_modes_passes_validation():
    """NPT runs in every precision mode (a batch refuses it): validation accepts it, so creation
    gets as far as the device (MTG_E_CUDA without a GPU, MTG_OK with one)."""
    s, c = W.argon(ncell=4)
    c.precision, c.ensemble = "fp64", "NPT"
    c.coulomb = "cutoff"
    try:
        E.Engine(s, c).close()
    except E.MTGError as err:
        assert err.code not in (UNSUPPORTED, INVALID), str(err)


def test_reference_mode_has_all_pairs_coulomb_only():
    s, c = W.argon(ncell=2)
    c.coulomb = "cutoff"
    code, msg = create_code(s, c)
    assert code == INVALID and "all-pairs" in msg


def test_all_pairs_coulomb_with_charges_in_production_modes():
    s, c = W.water(n_mol=8, L=12.0, seed=2)
    c.precision, c.coulomb = "mixed", "allpairs"
    code, msg = create_code(s, c)
    assert code == UNSUPPORTED and "all-pairs" in msg


def test_non_finite_positions():
    s, c = W.argon(ncell=2)
    s.r = s.r.copy()
    s.r[3, 1] = np.nan
    code, _ = create_code(s, c)
    assert code == NONFINITE


def test_non_positive_mass():
    s, c = W.argon(ncell=2)
    s.m = s.m.copy()
    s.m[0] = 0.0
    code, msg = create_code(s, c)
    assert code == INVALID and "mass" in msg


def test_non_positive_box():
    s, c = W.argon(ncell=2)
    s.box = np.array([s.box[0], 0.0, s.box[2]])
    code, msg = create_code(s, c)
    assert code == INVALID and "box" in msg


def batch_code(systems, c, **kw):
    from moltwister_gb300.batch import BatchEngine
    with pytest.raises(E.MTGError) as ei:
        BatchEngine(systems, c, **kw)
    return ei.value.code, str(ei.value)


def test_batch_needs_a_production_mode():
    a, c = W.argon(ncell=2, seed=1)
    b, _ = W.argon(ncell=3, seed=2)
    code, msg = batch_code([a, b], c)                     # the argon config is reference precision
    assert code == UNSUPPORTED and "batches" in msg


def test_batch_temperatures_and_cutoffs_are_checked():
    a, c = W.argon(ncell=2, seed=1)
    b, _ = W.argon(ncell=3, seed=2)
    c.precision = "mixed"
    code, msg = batch_code([a, b], c, temperatures=[120.0, -5.0])
    assert code == INVALID and "temperatures" in msg
    code, msg = batch_code([a, b], c, cutoffs=[c.cutoffradius, 2.0 * c.cutoffradius])
    assert code == INVALID and "cutoffs" in msg


def test_batch_topology_index_outside_its_replica():
    # a bond index in [n_r, N) exists in the merged system but would join atoms of two replicas
    w, c = W.water(n_mol=8, L=12.0, seed=2)
    a, _ = W.argon(ncell=2, seed=1)
    c.precision, c.coulomb, c.coulombcutoff = "mixed", "shifted", 5.0
    w.bonds = np.asarray(w.bonds).copy()
    w.bonds[0, 1] = w.n + 1
    code, msg = batch_code([w, a], c)
    assert code == INVALID and "replica 0" in msg and "outside" in msg
