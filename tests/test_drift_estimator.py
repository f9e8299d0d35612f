"""The NVE drift estimator of the Kob-Andersen benchmark (bench_kob_andersen._drift): slope of the
total energy per atom and kT against time, with a standard error from the fit of block means.
Synthetic energy series with a known slope and white noise; no GPU."""
import numpy as np

from moltwister_gb300.bench_kob_andersen import _drift


def _series(slope_kT_atom_ns, noise_kT_atom, n=4000, stride=20, dt_fs=0.5, atoms=1000, kT=0.75, seed=0):
    rng = np.random.default_rng(seed)
    steps = np.arange(n) * stride
    t_ns = steps * dt_fs * 1e-6
    E = atoms * kT * (slope_kT_atom_ns * t_ns + noise_kT_atom * rng.standard_normal(n))
    return list(zip(steps.tolist(), E.tolist())), atoms, kT, dt_fs, t_ns


def test_recovers_slope_within_its_standard_error():
    recs, n, kT, dt, t_ns = _series(3e-3, 2e-5)
    slope, se, noise = _drift(recs, n, kT, dt)
    assert abs(slope - 3e-3) < 4 * se
    assert abs(noise - 2e-5) < 0.1 * 2e-5


def test_standard_error_matches_white_noise_theory():
    # for white noise the slope's standard error is sigma / sqrt(sum (t - tbar)^2)
    ses = []
    for seed in range(8):
        recs, n, kT, dt, t_ns = _series(0.0, 2e-5, seed=seed)
        ses.append(_drift(recs, n, kT, dt)[1])
    theory = 2e-5 / np.sqrt(((t_ns - t_ns.mean()) ** 2).sum())
    assert 0.5 * theory < np.median(ses) < 2.0 * theory


def test_short_series_has_no_standard_error():
    recs, n, kT, dt, _ = _series(0.0, 1e-5, n=30)
    slope, se, noise = _drift(recs, n, kT, dt)
    assert se is None and slope is not None
    assert _drift(recs[:2], n, kT, dt) == (None, None, None)
