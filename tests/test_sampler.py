"""The keyed Poisson sampler and the project's exp/log (oracle statement):
accuracy against numpy/scipy and distributional checks."""
import math

import numpy as np
import pytest

from oracle_lib import oracle_lib


def test_exp_log_accuracy():
    L = oracle_lib()
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-40, 5, 2000), -rng.uniform(0, 10, 2000)])
    for x in xs:
        e = L.beep_oracle_exp(float(x))
        assert abs(e - math.exp(x)) <= 4e-16 * math.exp(x)
    ys = np.concatenate([rng.uniform(1e-6, 10, 2000), np.exp(rng.uniform(-300, 300, 2000))])
    for y in ys:
        lg = L.beep_oracle_log(float(y))
        assert abs(lg - math.log(y)) <= 4e-16 * max(1.0, abs(math.log(y)))


def test_log_factorial():
    L = oracle_lib()
    for k in list(range(0, 60)) + [100, 1000, 12345, 10 ** 6]:
        assert abs(L.beep_oracle_log_factorial(float(k)) - math.lgamma(k + 1)) <= 1e-13 * max(1.0, math.lgamma(k + 1))


@pytest.mark.parametrize("mean", [1e-4, 0.3, 2.5, 9.9, 10.0, 37.5, 400.0, 2.5e4])
def test_poisson_moments_and_distribution(mean):
    stats = pytest.importorskip("scipy.stats")
    L = oracle_lib()
    n = 20000
    x = np.array([L.beep_oracle_poisson(mean, 0xABCDEF0123456789, c % 997, 1, c // 997, 3) for c in range(n)])
    se = math.sqrt(mean / n)
    assert abs(x.mean() - mean) < 5 * se + 1e-12
    if mean > 0.01:
        assert abs(x.var() / mean - 1) < 6 * math.sqrt(2.0 / n) + 0.01
        # chi-square over well-populated bins
        lo, hi = int(max(0, mean - 4 * math.sqrt(mean))), int(mean + 4 * math.sqrt(mean)) + 1
        edges = np.arange(lo, hi + 1)
        obs = np.array([np.sum(x == k) for k in edges[:-1]])
        exp = n * stats.poisson.pmf(edges[:-1], mean)
        keep = exp > 20
        chi2 = np.sum((obs[keep] - exp[keep]) ** 2 / exp[keep])
        dof = max(1, keep.sum() - 1)
        assert stats.chi2.sf(chi2, dof) > 1e-4


def test_draws_are_a_function_of_the_counter():
    L = oracle_lib()
    a = [L.beep_oracle_poisson(3.3, 42, 7, tr, 11, 5) for tr in range(6)]
    b = [L.beep_oracle_poisson(3.3, 42, 7, tr, 11, 5) for tr in range(6)]
    c = [L.beep_oracle_poisson(3.3, 43, 7, tr, 11, 5) for tr in range(6)]
    assert a == b and a != c
