"""Short inference runs on top of the hot path, for the posterior-agreement
tests: the same algorithm driven by the plain FP64 form, the fast form or the
oracle, so that their posteriors can be compared.

* ``abc_smc``: ABC-SMC after ABCSMC::run (src/abcsmc.cc:26-123): generation 0
  samples the prior; each later generation draws a particle of the last one
  by weight, perturbs it with the multivariate normal of the last
  generation's weighted covariance (MVN::setup / MVN::propose,
  src/mvn.cc:39-80,277-292), keeps proposals inside the prior's bounds whose
  error function EF = -2L is below the last cut-off, and weights them with
  ABCSMC::calculate_particle_weight (src/abcsmc.cc:260-271); the cut-off of a
  generation is the cutoff_frac quantile of its EF (implement_cutoff_frac,
  src/abcsmc.cc:159-183) and the weights are normalised to mean one.  As on
  a GPU, proposals are simulated in batches: each round proposes as many
  candidates as the generation still lacks (at least a floor), rather than
  one at a time.
* ``pmcmc``: random-walk Metropolis-Hastings on the bootstrap particle
  filter's likelihood estimate (PMCMC::obs_prob, src/pmcmc.cc:180-268), with
  uniform priors.

Every random choice comes from numpy generators seeded per run, and every
simulation from the keyed variate streams (stream numbers fixed by the
round and candidate index), so a run is a deterministic function of its
seed and of the simulator it is given."""
from __future__ import annotations

import numpy as np

from beep_gb300 import capi, model_builder as mb, synth

PRIOR_LO = np.array([1.5, 2.0, 3.0])      # R0, 1/sigma, 1/gamma: the ABC-SMC workload's priors
PRIOR_HI = np.array([4.0, 6.0, 8.0])


def gpu_simulator(dm: capi.DeviceModel, m: capi.Model, w, form: int):
    """simulate(theta [n][3], seed, stream0) -> L [n] through the C ABI."""
    def simulate(theta, seed, stream0):
        tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, theta[:, 0], theta[:, 1], theta[:, 2])]
        n = len(theta)
        b = dm.simulate(capi.Batch(m, tabs, n, seed, group_of=np.arange(n), stream_of=stream0 + np.arange(n),
                                   form=form))
        return b.L.copy()
    return simulate


def oracle_simulator(m: capi.Model, w):
    from oracle_lib import oracle_simulate

    def simulate(theta, seed, stream0):
        tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, theta[:, 0], theta[:, 1], theta[:, 2])]
        n = len(theta)
        b = oracle_simulate(m, capi.Batch(m, tabs, n, seed, group_of=np.arange(n), stream_of=stream0 + np.arange(n)))
        return b.L.copy()
    return simulate


def weighted_cov(theta, w):
    """MVN::covariance_matrix with weights: sum_k w_k (x_k - mean)(x_k - mean)^T / sum w."""
    wn = w / w.sum()
    mu = (wn[:, None] * theta).sum(0)
    d = theta - mu
    return (wn[:, None, None] * d[:, :, None] * d[:, None, :]).sum(0)


def abc_smc(simulate, weights, N: int, generations: int, seed: int, cutoff_frac: float = 0.5,
            propsize: float = 1.0, min_round: int = 512):
    """Returns the generations: dicts of theta [n][3], EF [n], w [n] (mean 1) and EFcut."""
    rng = np.random.default_rng(seed)
    log_prior = -np.log(np.prod(PRIOR_HI - PRIOR_LO))
    gens = []
    want = int(N / cutoff_frac)
    # generation 0: the prior
    th = rng.uniform(PRIOR_LO, PRIOR_HI, (want, 3))
    EF = -2.0 * simulate(th, seed, 0)
    w = np.ones(want)
    for g in range(generations):
        if g > 0:
            last = gens[-1]
            cov = weighted_cov(last["theta"], last["w"])
            chol = np.linalg.cholesky(cov)
            inv_cov = np.linalg.inv(cov)
            p_sel = last["w"] / last["w"].sum()
            th_acc, EF_acc = [], []
            rnd = 0
            while sum(len(x) for x in th_acc) < want:
                n = max(min_round, want - sum(len(x) for x in th_acc))
                parents = rng.choice(len(p_sel), size=n, p=p_sel)
                prop = last["theta"][parents] + propsize * rng.standard_normal((n, 3)) @ chol.T
                ok = np.all((prop >= PRIOR_LO) & (prop <= PRIOR_HI), axis=1)
                prop = prop[ok]
                if len(prop):
                    ef = -2.0 * simulate(prop, seed + 1000 * g + rnd, 10 ** 6 * g + 10 ** 5 * rnd)
                    keep = ef < last["EFcut"]
                    th_acc.append(prop[keep])
                    EF_acc.append(ef[keep])
                rnd += 1
            # the generation holds exactly `want` accepted proposals (ABCSMC::run stops
            # proposing once the generation is full), in proposal order
            th = np.concatenate(th_acc)[:want]
            EF = np.concatenate(EF_acc)[:want]
            # calculate_particle_weight for the accepted samples (not normalised yet)
            w = weights(th, np.full(len(th), log_prior), last["theta"], last["w"], inv_cov, propsize)
        # implement_cutoff_frac: the cutoff_frac quantile; samples at or above it are dropped
        EFcut = np.sort(EF)[int(cutoff_frac * len(EF))]
        keep = EF < EFcut
        th, EF, w = th[keep], EF[keep], w[keep]
        gens.append({"theta": th, "EF": EF, "w": w / w.mean(), "EFcut": EFcut})
    return gens


def posterior_moments(theta, w):
    """Weighted mean, variance and effective sample size of each parameter."""
    wn = w / w.sum()
    mu = (wn[:, None] * theta).sum(0)
    var = (wn[:, None] * (theta - mu) ** 2).sum(0)
    ess = 1.0 / np.sum(wn ** 2)
    return mu, var, ess


def pmcmc(loglik, theta0, step, lo, hi, iters: int, seed: int):
    """Random-walk MH with uniform priors on [lo, hi]; loglik(theta, k) is the
    filter's estimate for iteration k.  Returns the chain [iters][d] and the
    acceptance rate."""
    rng = np.random.default_rng(seed)
    th = np.array(theta0, float)
    ll = loglik(th, 0)
    chain = np.zeros((iters, len(th)))
    acc = 0
    for k in range(iters):
        prop = th + step * rng.standard_normal(len(th))
        u = rng.random()
        if np.all((prop >= lo) & (prop <= hi)):
            llp = loglik(prop, k + 1)
            if np.log(u) < llp - ll:
                th, ll = prop, llp
                acc += 1
        chain[k] = th
    return chain, acc / iters


def batch_means_se(x, nbatch: int = 10):
    """Monte Carlo standard error of the mean of a correlated chain (batch means)."""
    n = len(x) // nbatch * nbatch
    b = x[:n].reshape(nbatch, -1).mean(1)
    return b.std(ddof=1) / np.sqrt(nbatch)


def c1_shaped(narea: int = 40, seed: int = 20260601):
    """The ABC-SMC workload's model at fewer areas (SEIR-H-D, 4 ages, dt 0.5,
    180 days, daily cases per area and age), observed data from one oracle
    simulation at R0 2.5, 1/sigma 4, 1/gamma 5 plus noise."""
    from oracle_lib import oracle_simulate
    w = synth.abc_smc_large(narea=narea, name=f"c1_{narea}")
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    t = [capi.Tables(x) for x in mb.param_tables_batch(w, [2.5], [4.0], [5.0])]
    truth = oracle_simulate(m0, capi.Batch(m0, t, 1, seed, want_transnum=True, want_pop_traj=True, want_L=False))
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], np.random.default_rng(seed))
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    return w, capi.Model(arr)
