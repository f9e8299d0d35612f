"""Failure and recovery paths of the engine, made to happen without faulting the GPU.

- List overflow: the neighbour lists start at a capacity of 1 entry per atom (the reference starts
  at 10, MDFFMatrices.cpp:246), overflow on the first build, grow (need + 10 in reference mode,
  MDFFMatrices.cpp:163-178; need + 25 % in the production modes) and the step or chunk is redone.
  The trajectory is bit-identical to a run that never overflowed.
- Bounded waits: with a wait limit of 0 polls every hand-over between the thermostat's warps gives
  up at once; the run returns MTG_E_TIMEOUT and the context runs normally again after the limit is
  restored and the state is set.
- Non-finite state: a momentum large enough that p^2/m overflows ends the run with
  MTG_E_NONFINITE at the first step end, not at the next output step.
"""
import numpy as np
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu

TIMEOUT, NONFINITE = -5, -7


@pytest.fixture(scope="module", autouse=True)
def built():
    from moltwister_gb300.build import build
    build()


def engine(s, cfg, **kw):
    from moltwister_gb300.engine import Engine
    return Engine(s, cfg, **kw)


def test_reference_list_overflow_regrows_and_redoes_the_step():
    s, cfg, d = G.load("argon500_nvt")
    runs = []
    for cap in (0, 1):
        cfg.initialmaxneighbours = cap
        e = engine(s, cfg)
        e.run(25)
        runs.append(e.get_state()[:2])
        e.close()
    (r0, p0), (r1, p1) = runs
    assert np.array_equal(r0, r1) and np.array_equal(p0, p1)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_production_list_overflow_regrows_and_redoes_the_chunk(prec):
    from moltwister_gb300 import workloads as W
    s, cfg = W.water(n_mol=216, L=W.water_box_length(216), seed=14, rc=6.0)
    cfg.precision, cfg.coulomb, cfg.coulombcutoff = prec, "shifted", 6.0
    runs = []
    for cap in (0, 1):
        cfg.initialmaxneighbours = cap
        e = engine(s, cfg)
        e.run(60, out_stride=20)
        runs.append(e.get_state()[:2])
        e.close()
    (r0, p0), (r1, p1) = runs
    assert np.array_equal(r0, r1) and np.array_equal(p0, p1)


def test_wait_limit_zero_times_out_and_the_context_recovers():
    from moltwister_gb300 import workloads as W
    from moltwister_gb300.engine import MTGError
    s, cfg = W.argon(ncell=5, seed=11, jitter=0.05)
    cfg.precision = "mixed"
    e = engine(s, cfg)
    r0, p0, th0 = e.get_state()
    e.set_wait_limit(0)
    with pytest.raises(MTGError) as ei:
        e.run(5)
    assert ei.value.code == TIMEOUT
    e.set_wait_limit(1 << 22)
    e.set_state(r=r0, p=p0, thermo=th0)
    recs = e.run(20, out_stride=10)
    r, p, _ = e.get_state()
    assert np.all(np.isfinite(r)) and np.all(np.isfinite(p))
    assert all(np.isfinite(x.T) and np.isfinite(x.U) for x in recs)


@pytest.mark.parametrize("prec,big", [("mixed", 1e30), ("fp64", 1e200)])
def test_non_finite_kinetic_energy_is_reported_at_the_step_end(prec, big):
    from moltwister_gb300 import workloads as W
    from moltwister_gb300.engine import MTGError
    s, cfg = W.argon(ncell=5, seed=11, jitter=0.05)
    cfg.precision = prec
    cfg.clipforces = False
    e = engine(s, cfg)
    r, p, th = e.get_state()
    p = p.copy()
    p[7] = [big, 0.0, 0.0]
    e.set_state(r=r, p=p, thermo=th)
    with pytest.raises(MTGError) as ei:
        e.run(50, out_stride=1000)          # no output step inside the run
    assert ei.value.code == NONFINITE


@pytest.mark.parametrize("prec", ["reference", "mixed"])
def test_output_stream_and_early_stop(prec):
    """Output steps stream through the pinned double buffer while the next chunk runs: the records
    carry the positions and momenta of their own step (equal to a run that ends there), and a
    callback that asks to stop leaves the state after its step even though the next chunk had
    already been queued."""
    from moltwister_gb300 import workloads as W
    s, cfg = W.argon(ncell=5, seed=11, jitter=0.05)
    cfg.precision = prec
    e1 = engine(s, cfg)
    recs = e1.run(100, out_stride=10, callback=lambda rec: rec.step >= 50)
    assert [r.step for r in recs] == [0, 10, 20, 30, 40, 50]
    r1, p1, _ = e1.get_state()
    e2 = engine(s, cfg)
    recs2 = e2.run(51, out_stride=10)
    r2, p2, _ = e2.get_state()
    assert np.array_equal(r1, r2) and np.array_equal(p1, p2)
    for a, b in zip(recs, recs2):
        assert a.step == b.step and np.array_equal(a.r, b.r) and np.array_equal(a.p, b.p) and a.U == b.U
    assert np.array_equal(recs[-1].r, r2) and np.array_equal(recs[-1].p, p2)
