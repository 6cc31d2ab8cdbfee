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


@pytest.mark.parametrize("kind,batched,traffic", [("abc_smc", True, True), ("abc_smc", False, True),
                                                  ("precision", True, False)])
def test_bench_reads_the_committed_profiles(kind, batched, traffic):
    """The per-particle figures the bench's rooflines read from the committed ncu
    summaries (warp instructions per launch; DRAM bytes where the capture's traffic
    scales with the particles) are present and positive."""
    inst = bench.profile_figure(kind, batched, "warp_instructions_per_particle")
    assert inst is not None and inst > 0
    dram = bench.profile_traffic(kind, 16384, batched)
    assert (dram is not None and dram > 0) if traffic else True


def test_issue_roofline_arithmetic():
    """Issue roofline: warp instructions per launch over 152 SMs x 4 schedulers x the
    sampled clock; a launch issuing exactly that many in one second is at 1.0."""
    per = bench.profile_figure("abc_smc", True, "warp_instructions_per_particle")
    P = 1000
    peak = 152 * 4 * 2070e6
    r = bench.issue_roofline("abc_smc", P, per * P / peak, {"sm_mhz": 2070.0}, True)
    assert abs(r["frac"] - 1.0) < 1e-9
    assert r["source"].startswith("profiles/")
