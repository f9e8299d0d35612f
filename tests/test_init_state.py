"""Initial momenta and chain state (mtg_draw_initial_state / mtg_init_state).

The reference mode is pinned to the reference's own CSimulationBox constructor run after
srand(seed) (tests/golden/init_states.npz, from oracle/ref/harness.cpp `init`): momenta, thermostat
chain positions and momenta, barostat chain and barostat momentum, bit for bit.  The draw runs on
the host, so these tests need no GPU; one GPU test sets a drawn state on a context and runs it."""
import json
import os

import numpy as np
import pytest

from moltwister_gb300 import engine as E
from moltwister_gb300 import workloads as W
from moltwister_gb300.system import MDConfig

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "init_states.npz")
CASES = ["chains108_seed1", "chains108_seed12345", "argon500_seed1", "water648_npt_seed7"]


@pytest.fixture(scope="module", autouse=True)
def built():
    from moltwister_gb300.build import build
    build()


def fixture_case(name):
    d = np.load(GOLDEN)
    m = d[f"{name}__m"]
    mobile = d[f"{name}__mobile"].astype(bool)
    cfg = MDConfig(**json.loads(str(d[f"{name}__cfg"])))
    s, _ = W.argon(ncell=1, seed=0)             # any system: the draw reads n, masses and mobility
    n = m.shape[0]
    s.ids, s.r, s.q, s.m, s.mobile = ["Ar"] * n, np.zeros((n, 3)), np.zeros(n), m, mobile
    s.mol = np.arange(n, dtype=np.int32)
    return s, cfg, int(d[f"{name}__seed"]), {k: d[f"{name}__{k}"] for k in ("init_p", "init_nhT", "init_nhP", "init_peps")}


@pytest.mark.parametrize("name", CASES)
def test_reference_draw_matches_the_reference_constructor(name):
    s, cfg, seed, ref = fixture_case(name)
    p, th = E.draw_initial_state(s, cfg, seed, "reference")
    assert np.array_equal(p, ref["init_p"])
    assert np.array_equal(th.eta, ref["init_nhT"][0]) and np.array_equal(th.peta, ref["init_nhT"][1])
    assert np.array_equal(th.etaP, ref["init_nhP"][0]) and np.array_equal(th.petaP, ref["init_nhP"][1])
    assert th.p_eps == ref["init_peps"][0]


def test_reference_draw_scales_with_unit_masses():
    """The reference scales the momenta before it copies the masses in (SimulationBox.cpp:53-96),
    so sum p^2 (not sum p^2/m) over 3N equals kT."""
    s, cfg, seed, _ = fixture_case("chains108_seed1")
    p, _ = E.draw_initial_state(s, cfg, seed, "reference")
    kT = cfg.temperature / 120.272
    assert abs((p * p).sum() / (3 * s.n) - kT) < 1e-12 * kT
    assert np.all(p[~s.mobile] == 0.0)


def test_maxwell_draw():
    s, cfg = W.chains(n_chain=27, L=24.0, seed=15, immobile_every=7)
    p, th = E.draw_initial_state(s, cfg, 5, "maxwell")
    p2, _ = E.draw_initial_state(s, cfg, 5, "maxwell")
    p3, _ = E.draw_initial_state(s, cfg, 6, "maxwell")
    assert np.array_equal(p, p2) and not np.array_equal(p, p3)
    kT = cfg.temperature / 120.272
    assert abs((p * p / s.m[:, None]).sum() / (3 * s.n) - kT) < 1e-12 * kT
    assert np.all(p[~s.mobile] == 0.0)
    assert np.abs(p[s.mobile].sum(0)).max() < 1e-9 * np.abs(p).max()
    assert len(th.eta) == cfg.temperaturenhlen and np.all((th.eta >= 0) & (th.eta < 1))


def test_bad_mode_is_rejected():
    s, cfg = W.argon(ncell=2)
    with pytest.raises(KeyError):
        E.draw_initial_state(s, cfg, 1, "uniform")


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["reference", "mixed"])
def test_init_state_sets_the_drawn_state(prec):
    s, cfg = W.argon(ncell=5, seed=11, jitter=0.05)
    cfg.precision = prec
    e = E.Engine(s, cfg)
    e.init_state(3, "reference")
    r, p, th = e.get_state()
    pd, thd = E.draw_initial_state(s, cfg, 3, "reference")
    if prec == "mixed":   # momenta kept as double-float pairs (48 significant bits)
        assert np.allclose(p, pd, rtol=1e-14, atol=0.0)
    else:
        assert np.array_equal(p, pd)
    assert np.array_equal(th.eta, thd.eta) and np.array_equal(th.peta, thd.peta)
    recs = e.run(20, out_stride=10)
    assert all(np.isfinite(x.T) for x in recs)
