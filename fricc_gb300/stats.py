"""Statistics of stochastic energy traces: fri-cc's ``mcmc_std``.

The reference reports the error bar of a correlated FRI energy trace as
``mcmc_std(vals)`` (fricc/__init__.py:8-11): sqrt(tau / n * var(vals)) with tau
the integrated autocorrelation time from ``emcee.autocorr.integrated_time``
(emcee 3, third party, unpinned; not installed here).  That estimator is
Sokal's automatic windowing (A. Sokal, "Monte Carlo Methods in Statistical
Mechanics", 1989; as used by Goodman and Weare, 2010, and documented by
emcee), restated here from the method:

* rho(t), the normalised autocorrelation of the mean-subtracted trace, from
  an FFT zero-padded to twice the next power of two of n (no wrap-around);
  walkers (a second axis) average their rho;
* tau(M) = 1 + 2 sum_{t=1..M} rho(t);
* the window is the first M with M >= c tau(M) (c = 5), else the last lag;
* a trace shorter than tol * tau (tol = 50) is too short to trust:
  ``AutocorrError`` unless ``quiet``, then a warning.
"""
from __future__ import annotations

import warnings

import numpy as np


class AutocorrError(Exception):
    """The trace is shorter than tol integrated autocorrelation times."""

    def __init__(self, tau, msg):
        self.tau = tau
        super().__init__(msg)


def _pow2_at_least(n: int) -> int:
    p = 1
    while p < n:
        p <<= 1
    return p


def autocorr_1d(x) -> np.ndarray:
    """rho(t), t = 0..n-1, of a 1-D trace (rho(0) = 1)."""
    x = np.asarray(x, dtype=np.float64)
    if x.ndim != 1:
        raise ValueError("autocorr_1d takes a 1-D trace")
    n = x.size
    size = 2 * _pow2_at_least(n)
    y = np.fft.rfft(x - x.mean(), n=size)
    acov = np.fft.irfft(y * np.conj(y), n=size)[:n]
    return acov / acov[0]


def _window(taus: np.ndarray, c: float) -> int:
    ok = np.arange(taus.size) < c * taus
    return int(np.argmin(ok)) if not ok.all() else taus.size - 1


def integrated_time(x, c: float = 5, tol: float = 50, quiet: bool = False, has_walkers: bool = True) -> np.ndarray:
    """Integrated autocorrelation time per parameter.

    ``x`` is (steps,), (steps, walkers) -- or (steps, params) with
    ``has_walkers=False`` -- or (steps, walkers, params)."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    if x.ndim == 1:
        x = x[:, None, None]
    elif x.ndim == 2:
        x = x[:, :, None] if has_walkers else x[:, None, :]
    if x.ndim != 3:
        raise ValueError("integrated_time takes (steps,), (steps, walkers) or (steps, walkers, params)")
    n_t, n_w, n_d = x.shape
    tau = np.empty(n_d)
    for d in range(n_d):
        rho = sum(autocorr_1d(x[:, k, d]) for k in range(n_w)) / n_w
        taus = 2.0 * np.cumsum(rho) - 1.0
        tau[d] = taus[_window(taus, c)]
    if np.any(tol * tau > n_t):
        msg = (f"the trace ({n_t} steps) is shorter than {tol} integrated autocorrelation times "
               f"(tau = {tau}); a longer trace is needed for a reliable estimate")
        if not quiet:
            raise AutocorrError(tau, msg)
        warnings.warn(msg)
    return tau


def mcmc_std(vals, quiet: bool = False):
    """(error bar of the trace's mean, tau) = (sqrt(tau / n var(vals)), tau)
    (fricc/__init__.py:8-11; ``quiet`` lets a short trace warn instead of raise)."""
    vals = np.asarray(vals, dtype=np.float64)
    tau = integrated_time(vals, quiet=quiet)[0]
    return np.sqrt(tau / vals.size * np.var(vals)), tau
