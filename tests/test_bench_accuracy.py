"""The bench's FP64 scorer of a fast trajectory (the log-likelihood error it
reports for the fast form) against the oracle's own FP64 log-likelihoods."""
import numpy as np
import pytest

import bench
from beep_gb300 import capi
from golden_util import load
from oracle_lib import oracle_simulate


@pytest.mark.parametrize("name", ["c0_sim", "features_sim"])
def test_fp64_scorer_matches_oracle(name):
    b, m, tabs, seed = load(name)
    o = oracle_simulate(m, capi.Batch(m, tabs, 4, seed, want_transnum=True))
    for k in range(4):
        l64 = bench.fp64_loglik_of_trajectory(m, o.transnum[k])
        assert abs(l64 - o.L[k]) <= 1e-12 * abs(o.L[k])


def test_fp64_scorer_declines_other_observation_models():
    b, m, tabs, seed = load("obsmodel_sim")
    o = oracle_simulate(m, capi.Batch(m, tabs, 1, seed, want_transnum=True))
    assert bench.fp64_loglik_of_trajectory(m, o.transnum[0]) is None
