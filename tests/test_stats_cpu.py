"""fri-cc's mcmc_std (fricc/__init__.py:8-11) and the integrated
autocorrelation time it takes from emcee, restated in fricc_gb300.stats."""
import numpy as np
import pytest

from fricc_gb300 import stats


def _ar1(phi, n, seed, walkers=None):
    rng = np.random.default_rng(seed)
    shape = (n,) if walkers is None else (n, walkers)
    e = rng.standard_normal(shape)
    x = np.empty(shape)
    x[0] = e[0] / np.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    return x


def test_autocorr_matches_direct_sum():
    x = np.random.default_rng(3).standard_normal(257).cumsum()
    y = x - x.mean()
    direct = np.array([np.dot(y[: y.size - t], y[t:]) for t in range(y.size)])
    np.testing.assert_allclose(stats.autocorr_1d(x), direct / direct[0], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.8])
def test_ar1_tau_matches_theory(phi):
    # tau of an AR(1) trace is (1 + phi) / (1 - phi)
    x = _ar1(phi, 200_000, seed=11)
    tau = stats.integrated_time(x)[0]
    assert abs(tau - (1 + phi) / (1 - phi)) < 0.08 * (1 + phi) / (1 - phi)


def test_window_rule():
    # taus = 2 cumsum(rho) - 1; the window is the first M with M >= c tau(M)
    rho = np.array([1.0, 0.5, 0.25, 0.125, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0])
    taus = 2 * np.cumsum(rho) - 1
    # taus = 1, 2, 2.5, 2.75, 2.75, ...: with c = 5 no lag reaches 5 tau (13 < 13.75),
    # so the window is the last lag; with c = 1 it is M = 3 (3 >= 2.75)
    assert stats._window(taus, 5) == taus.size - 1
    assert stats._window(taus, 1) == 3


def test_walkers_average_and_shapes():
    x = _ar1(0.5, 20_000, seed=5, walkers=4)
    t_w = stats.integrated_time(x)                         # (steps, walkers)
    t_3 = stats.integrated_time(x[:, :, None])            # (steps, walkers, params)
    t_p = stats.integrated_time(x, has_walkers=False)      # (steps, params): one tau per column
    assert t_w.shape == (1,) and t_3.shape == (1,) and t_p.shape == (4,)
    assert t_w[0] == t_3[0]
    assert abs(t_w[0] - 3.0) < 0.3 and np.all(np.abs(t_p - 3.0) < 0.6)
    with pytest.raises(ValueError):
        stats.integrated_time(np.zeros((4, 4, 4, 4)))


def test_short_trace_raises_or_warns():
    x = _ar1(0.9, 200, seed=1)
    with pytest.raises(stats.AutocorrError) as ei:
        stats.integrated_time(x)
    assert ei.value.tau.shape == (1,)
    with pytest.warns(UserWarning):
        stats.integrated_time(x, quiet=True)


def test_mcmc_std_white_noise_and_ar1():
    x = np.random.default_rng(7).standard_normal(50_000)
    err, tau = stats.mcmc_std(x)
    assert abs(tau - 1) < 0.05
    assert abs(err - np.sqrt(np.var(x) / x.size)) < 0.05 * np.sqrt(np.var(x) / x.size)
    y = _ar1(0.8, 100_000, seed=2)
    err, tau = stats.mcmc_std(y)
    assert err == pytest.approx(np.sqrt(tau / y.size * np.var(y)), rel=0, abs=0)
