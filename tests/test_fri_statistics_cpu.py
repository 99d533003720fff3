"""Statistical properties of FRI compression: the checks of the reference's
fricc/tests/test_fri_utils.py restated as tests, run on the oracle (CPU).
The GPU compressions are bit-identical to the oracle's (tests/test_gpu_compress.py,
tests/test_gpu_pivotal.py), so these properties carry over to them.

* the exactly kept set D and the remaining norm R (``find_d_largest``,
  test_fri_utils.py:30-46);
* the probability vector p_i = |x_i| m' / R off D (``make_p``, :48-54): every
  sampled value is x_i / p_i, of magnitude R / m';
* unbiasedness: the average of many compressions converges to x (the
  reference's script, :85-176, averages 10^4 systematic compressions and fits
  the error's power law).
"""
import numpy as np
import pytest


def find_d_largest(n_sample, x):
    """The reference test's plain restatement of get_d_largest
    (test_fri_utils.py:30-46): walk |x| in descending order, keep x_(d) while
    (n_sample - d) |x_(d)| >= R - |x_(d)|."""
    R = float(np.sum(np.abs(x)))
    D = []
    for idx in np.argsort(-np.abs(x), kind="stable")[:n_sample]:
        xi = abs(x[idx])
        if (n_sample - len(D)) * xi >= R - xi:
            D.append(int(idx))
            R -= xi
        else:
            break
    return D, R


def _vectors():
    rng = np.random.default_rng(20)
    n = 20000
    flat = rng.random(n) - rng.random(n)                      # D empty for m << n
    heavy = (rng.random(n) - 0.5) * np.logspace(1, -10, n)    # heavy tail: D non-empty for m >= 700
    return {"flat": flat, "heavy": heavy}


@pytest.mark.parametrize("name", ["flat", "heavy"])
@pytest.mark.parametrize("m", [50, 700, 4000])
def test_d_largest_matches_restatement(oracle, name, m):
    x = _vectors()[name]
    D, R = oracle.get_d_largest(x, m)
    D_ref, R_ref = find_d_largest(m, x)
    assert list(D) == D_ref
    assert R == pytest.approx(R_ref, rel=1e-12)
    if name == "heavy" and m >= 700:
        assert len(D) > 0


@pytest.mark.parametrize("name", ["flat", "heavy"])
def test_sampled_values_are_x_over_p(oracle, name):
    """Off D, a kept value is x_i / p_i with p_i = |x_i| m' / R <= 1: its
    magnitude is R / m' and its sign x_i's; D keeps x_i exactly."""
    x = _vectors()[name]
    m = 700
    idx, val, nd = oracle.fri_compression(x, m, rn=0.375)
    D, R = oracle.get_d_largest(x, m)
    mp = m - nd
    assert nd == len(D) and np.array_equal(idx[:nd], D)
    assert np.array_equal(val[:nd], x[idx[:nd]])
    S = idx[nd:]
    assert np.all(np.diff(S) > 0) and not np.isin(S, D).any()
    p = np.abs(x[S]) / R * mp
    assert np.all(p <= 1.0)
    np.testing.assert_allclose(np.abs(val[nd:]), R / mp, rtol=1e-13)
    assert np.array_equal(np.sign(val[nd:]), np.sign(x[S]))


def _dense(idx, val, n):
    out = np.zeros(n)
    out[idx] = val
    return out


def test_systematic_unbiased_over_its_one_uniform(oracle):
    """Systematic resampling uses one uniform rn: over rn in [0, 1) each i off
    D is kept with probability exactly p_i.  K evenly spaced rn (midpoints)
    therefore keep i a fraction of times within 2/K of p_i, so the average
    is within (2/K) R/m' of x, element by element; D is exact every time."""
    x = _vectors()["heavy"][:4000]
    m, K = 400, 500
    acc = np.zeros(x.size)
    for k in range(K):
        idx, val, nd = oracle.fri_compression(x, m, rn=(k + 0.5) / K)
        acc += _dense(idx, val, x.size)
    D, R = oracle.get_d_largest(x, m)
    bound = 2.0 / K * R / (m - len(D))
    err = np.abs(acc / K - x)
    assert np.all(err <= bound * (1 + 1e-9) + 1e-15 * np.abs(x))
    assert np.all(err[D] <= 1e-12 * np.abs(x[D]))


def test_systematic_average_error_power_law(oracle):
    """The reference's experiment (test_fri_utils.py:85-176) on a smaller
    vector: the L1 error of the running average of compressions with random
    rn falls like K^b, with b near the Monte-Carlo -1/2 (systematic
    resampling is at least that good)."""
    rng = np.random.default_rng(20)
    x = rng.random(5000) - rng.random(5000)
    m, K = 500, 400
    acc = np.zeros(x.size)
    err = np.empty(K)
    for k in range(K):
        idx, val, _ = oracle.fri_compression(x, m, rn=float(rng.random()))
        acc += _dense(idx, val, x.size)
        err[k] = np.abs(x - acc / (k + 1)).sum() / np.abs(x).sum()
    ks = np.arange(1, K + 1)
    b = np.polyfit(np.log(ks[9:]), np.log(err[9:]), 1)[0]
    assert -1.2 < b < -0.4, b
    assert err[-1] < err[0] / 10


def test_pivotal_unbiased(oracle):
    """Pivotal sampling keeps exactly m' distinct indices off D, each with
    probability p_i: over K independent draws the average of the compressions
    is within 5 standard errors of x for every element (the value kept is
    x_i / p_i with probability p_i, so its variance is x_i^2 (1 - p_i) / p_i)."""
    rng = np.random.default_rng(7)
    x = (rng.random(300) - 0.5) * np.logspace(0, -3, 300)
    m, K = 60, 600
    D, R = oracle.get_d_largest(x, m)
    mp = m - len(D)
    acc = np.zeros(x.size)
    for _ in range(K):
        idx, val, nd, used = oracle.fri_compression_pivotal(x, m, draws=rng.random(2 * x.size + 8))
        assert nd == len(D) and len(np.unique(idx)) == m
        acc += _dense(idx, val, x.size)
    p = np.abs(x) / R * mp
    p[D] = 1.0
    se = np.abs(x) * np.sqrt((1 - p) / p / K)
    assert np.all(np.abs(acc / K - x) <= 5 * se + 1e-13 * np.abs(x))
