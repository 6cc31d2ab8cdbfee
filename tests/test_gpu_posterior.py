"""Posterior agreement from full inference runs (short ones): the same ABC-SMC
and PMCMC algorithms driven by the oracle, the plain FP64 form and the fast
form give the same posterior means and variances within Monte Carlo error.

* ABC-SMC (src/abcsmc.cc:26-123): three generations of 2048 particles on the
  ABC-SMC workload's model at 40 areas x 4 ages (dt 0.5, 180 days, daily
  cases per area and age), weights from beep_abcsmc_weights (GPU runs) or
  the oracle's FP64 weights.  The plain form's first generation is the
  oracle's, EF for EF.
* PMCMC (src/pmcmc.cc:33-114, 180-268): 500 random-walk Metropolis-Hastings
  iterations on the 10-area x 3-age model, the likelihood estimated by the
  bootstrap particle filter (256 particles, sections of 28 steps) at inverse
  temperature invT = 0.1 (the reference's tempered PMCMC, invT of src/pmcmc.cc:24,230-235:
  at invT = 1 the estimate's standard deviation is ~30 nats with 256
  particles and no chain of this length mixes; at 0.1 it is ~0.8).  The
  plain form's chain is the oracle's chain, iteration for iteration; the
  fast form's chain agrees in posterior mean (batch-means standard errors)
  and variance."""
import numpy as np
import pytest

from beep_gb300 import capi, model_builder as mb, synth
from inference_loops import (abc_smc, batch_means_se, c1_shaped, gpu_simulator, oracle_simulator, pmcmc,
                             posterior_moments)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    return capi.lib()


def _agree(mu1, var1, ess1, mu2, var2, ess2, what):
    se = np.sqrt(var1 / ess1 + var2 / ess2)
    z = np.abs(mu1 - mu2) / se
    assert np.all(z < 4.0), f"{what}: posterior means differ by {z} standard errors"
    lr = np.abs(np.log(var1 / var2))
    tol = 4.0 * np.sqrt(2.0 / ess1 + 2.0 / ess2)
    assert np.all(lr < tol), f"{what}: posterior variances differ: log ratio {lr} (allowed {tol})"


def test_abc_smc_posteriors_agree(built):
    from oracle_lib import oracle_abcsmc_weights
    w, m = c1_shaped(40)
    dm = capi.DeviceModel(m)
    runs = {
        "oracle": abc_smc(oracle_simulator(m, w), oracle_abcsmc_weights, 2048, 3, seed=77),
        "plain": abc_smc(gpu_simulator(dm, m, w, capi.FORM_PLAIN_FP64), capi.abcsmc_weights, 2048, 3, seed=77),
        "fast": abc_smc(gpu_simulator(dm, m, w, capi.FORM_FAST), capi.abcsmc_weights, 2048, 3, seed=77),
    }
    dm.close()
    # generation 0 is the prior sample: the plain form's EF are the oracle's
    np.testing.assert_allclose(runs["plain"][0]["EF"], runs["oracle"][0]["EF"], rtol=1e-12)
    final = {k: posterior_moments(g[-1]["theta"], g[-1]["w"]) for k, g in runs.items()}
    for k, g in runs.items():
        assert len(g[-1]["theta"]) == 2048
        assert final[k][2] > 200, (k, final[k][2])             # effective sample size
        # the cut-off falls from generation to generation, and the posterior of R0 (the
        # parameter daily cases identify; prior U(1.5, 4)) contracts to under 0.6 of the
        # prior variance (two oracle runs of other seeds: 0.42-0.47)
        assert all(a["EFcut"] > b["EFcut"] for a, b in zip(g, g[1:])), k
        assert final[k][1][0] < 0.6 * 2.5 ** 2 / 12, (k, final[k][1])
    _agree(*final["plain"], *final["oracle"], "plain vs oracle")
    _agree(*final["fast"], *final["plain"], "fast vs plain")
    _agree(*final["fast"], *final["oracle"], "fast vs oracle")


def test_pmcmc_chains_agree(built):
    from oracle_lib import oracle_pf
    w = synth.seir_hd_small()
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    dm0 = capi.DeviceModel(m0)
    truth = dm0.simulate(capi.Batch(m0, [capi.Tables(mb.param_tables(w))], 1, 4242, want_transnum=True,
                                    want_pop_traj=True, want_L=False))
    dm0.close()
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], np.random.default_rng(4243))
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    m = capi.Model(arr)
    S = m.ndivision
    sections = [(a, min(a + 28, S)) for a in range(0, S, 28)]
    N = 256
    invT = 0.1
    lo, hi = np.array([0.5, 2.0]), np.array([2.0, 6.0])          # R(t) scale, 1/sigma
    step = np.array([0.06, 0.7])                                 # ~30% acceptance

    def tables(th):
        return capi.Tables(mb.param_tables(w, sigma_inv=float(th[1]), R_scale=float(th[0])))

    dm = capi.DeviceModel(m)

    def gpu_ll(form):
        return lambda th, k: dm.pf_loglik(tables(th), N, 9000 + k, k, invT, sections, form=form)[0]

    def oracle_ll(th, k):
        return oracle_pf(m, tables(th), N, 9000 + k, k, invT, sections)[0]

    th0 = np.array([1.0, 4.0])
    iters = 500
    chains = {"plain": pmcmc(gpu_ll(capi.FORM_PLAIN_FP64), th0, step, lo, hi, iters, seed=5),
              "oracle": pmcmc(oracle_ll, th0, step, lo, hi, iters, seed=5),
              "fast": pmcmc(gpu_ll(capi.FORM_FAST), th0, step, lo, hi, iters, seed=5)}
    dm.close()
    # the plain form's filter is the oracle's filter: the same chain
    np.testing.assert_allclose(chains["plain"][0], chains["oracle"][0], rtol=1e-12)
    burn = 100
    mom = {}
    for k, (c, acc) in chains.items():
        assert 0.05 < acc < 0.9, (k, acc)
        x = c[burn:]
        se = np.array([batch_means_se(x[:, j]) for j in range(x.shape[1])])
        mom[k] = (x.mean(0), x.var(0), se)
    for a, b in (("fast", "plain"), ("fast", "oracle")):
        z = np.abs(mom[a][0] - mom[b][0]) / np.sqrt(mom[a][2] ** 2 + mom[b][2] ** 2)
        assert np.all(z < 4.0), (a, b, z, mom[a][0], mom[b][0])
        # variances: within a factor three (a short, autocorrelated chain estimates them loosely)
        assert np.all(np.abs(np.log(mom[a][1] / mom[b][1])) < np.log(3.0)), (a, b, mom[a][1], mom[b][1])
