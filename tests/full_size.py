"""The two large workloads at their full per-particle size, with observed data,
for the parity tests:

* ``abc_smc``: 150 areas x 4 ages, dt 0.5 day, 180 days (360 steps), daily
  cases per area and age (108,000 observations); the ABC-SMC generation's
  model;
* ``precision``: 350 areas x 10 ages, dt 0.25 day, 365 days (1460 steps),
  dense gravity mixing with long-range entries, stepped age-mixing factors,
  a 20-knot R(t) and two area covariates; daily cases and weekly deaths per
  area; the PMCMC precision model.

The observed data are one oracle simulation at the true parameters plus
normal noise of variance max(count, 5) (so no GPU is needed to make them)."""
from __future__ import annotations

import functools

import numpy as np

from beep_gb300 import capi, model_builder as mb, synth


@functools.lru_cache(maxsize=None)
def workload(kind: str, seed: int = 20260501):
    from oracle_lib import oracle_simulate
    w = synth.abc_smc_large() if kind == "abc_smc" else synth.precision_large()
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    t_true = capi.Tables(mb.param_tables(w))
    truth = oracle_simulate(m0, capi.Batch(m0, [t_true], 1, seed ^ 0x5EED, want_transnum=True, want_pop_traj=True,
                                           want_L=False))
    rng = np.random.default_rng(seed)
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], rng)
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    return w, capi.Model(arr), t_true


def prior_tables(w, n: int, seed: int):
    """n parameter sets from the ABC-SMC priors (R0, 1/sigma, 1/gamma)."""
    R0, si, gi = synth.abc_smc_priors(np.random.default_rng(seed), n)
    return [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
