"""ABC-SMC importance weights (src/abcsmc.cc:260-283): GPU kernel vs the
oracle's FP64 restatement.  Tolerance: 1e-5 relative (FP32 kernel terms,
compensated sums, FP64 normalisation)."""
import numpy as np
import pytest

from beep_gb300 import capi
from oracle_lib import oracle_abcsmc_weights


def generation(rng, nnew, nlast, nvar=3):
    # R0 U(1.5,4), 1/sigma U(2,6), 1/gamma U(3,8): the ABC-SMC workload's priors
    lo, hi = np.array([1.5, 2.0, 3.0]), np.array([4.0, 6.0, 8.0])
    tl = rng.uniform(lo, hi, (nlast, nvar))
    wl = rng.uniform(0.2, 2.0, nlast)
    tn = np.clip(tl[rng.integers(0, nlast, nnew)] + rng.normal(0, 0.2, (nnew, nvar)), lo, hi)
    # the weighted sample covariance needs more particles than parameters
    cov = np.cov(tl.T, aweights=wl) if nlast > nvar else np.diag(((hi - lo) / 4) ** 2)
    ic = np.linalg.inv(cov)
    lp = np.full(nnew, -np.log(np.prod(hi - lo)))
    return tn, lp, tl, wl, ic


def test_oracle_weights_match_direct_formula():
    rng = np.random.default_rng(3)
    tn, lp, tl, wl, ic = generation(rng, 20, 30)
    w = oracle_abcsmc_weights(tn, lp, tl, wl, ic, 1.5, normalise=False)
    for i in range(20):
        d = (tn[i] - tl) / 1.5
        q = np.einsum("jv,vu,ju->j", d, ic, d)
        assert abs(w[i] - np.exp(lp[i]) / np.sum(wl * np.exp(-0.5 * q))) <= 1e-12 * w[i]


@pytest.mark.gpu
@pytest.mark.parametrize("nnew,nlast", [(1, 1), (300, 257), (4096, 4096)])
def test_gpu_weights_match_oracle(nnew, nlast):
    from beep_gb300 import build
    build.build()
    rng = np.random.default_rng(nnew + nlast)
    tn, lp, tl, wl, ic = generation(rng, nnew, nlast)
    g = capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.3)
    o = oracle_abcsmc_weights(tn, lp, tl, wl, ic, 1.3)
    assert np.all(np.isfinite(o)) and np.all(o > 0)
    np.testing.assert_allclose(g, o, rtol=1e-5)


def _reference_case():
    from beep_gb300 import bundle
    import os
    b = bundle.read_bundle(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c0_abcw.bnd"))
    return ([np.asarray(b["abc." + k]) for k in ("theta_new", "logprior_new", "theta_last", "w_last", "inv_cov")],
            float(np.asarray(b["abc.size"]).ravel()[0]), np.asarray(b["abc.w"]), np.asarray(b["abc.w_norm"]))


def test_oracle_weights_match_reference():
    """The oracle against the reference's own ABCSMC::calculate_particle_weight
    and normalise_particle_weights (weighted MVN of 40 samples of the 10-area
    model's 12 free parameters, 24 new samples; tests/golden/c0_abcw.bnd)."""
    args, size, w_ref, wn_ref = _reference_case()
    np.testing.assert_allclose(oracle_abcsmc_weights(*args, size, normalise=False), w_ref, rtol=1e-12)
    np.testing.assert_allclose(oracle_abcsmc_weights(*args, size, normalise=True), wn_ref, rtol=1e-12)


@pytest.mark.gpu
def test_gpu_weights_match_reference():
    from beep_gb300 import build
    build.build()
    args, size, w_ref, wn_ref = _reference_case()
    np.testing.assert_allclose(capi.abcsmc_weights(*args, size, normalise=False), w_ref, rtol=1e-5)
    np.testing.assert_allclose(capi.abcsmc_weights(*args, size, normalise=True), wn_ref, rtol=1e-5)


def _logsumexp_weights(tn, lp, tl, wl, ic, size):
    """FP64 weights through a log-sum-exp (no underflow), normalised to mean 1."""
    out = np.zeros(len(tn))
    for i in range(len(tn)):
        d = (tn[i] - tl) / size
        x = np.log(wl) - 0.5 * np.einsum("jv,vu,ju->j", d, ic, d)
        m = x.max()
        out[i] = lp[i] - (m + np.log(np.exp(x - m).sum()))
    w = np.exp(out - out.max())
    return w / w.mean()


@pytest.mark.gpu
def test_gpu_weights_large_offsets():
    """Parameters of magnitude 1e3 with a spread of 1e-2: the differences are
    formed from values centred on the last generation's mean, so FP32 keeps
    the 1e-5 tolerance."""
    from beep_gb300 import build
    build.build()
    rng = np.random.default_rng(11)
    nvar, nnew, nlast = 3, 300, 400
    tl = 1000.0 + rng.normal(0.0, 0.01, (nlast, nvar))
    wl = rng.uniform(0.2, 2.0, nlast)
    tn = tl[rng.integers(0, nlast, nnew)] + rng.normal(0, 0.003, (nnew, nvar))
    ic = np.linalg.inv(np.cov(tl.T, aweights=wl))
    lp = np.zeros(nnew)
    g = capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.0)
    o = oracle_abcsmc_weights(tn, lp, tl, wl, ic, 1.0)
    np.testing.assert_allclose(g, o, rtol=1e-5)


@pytest.mark.gpu
def test_gpu_weights_where_fp32_terms_underflow():
    """New particles about 12 standard deviations from every previous one:
    quadratic forms of a few hundred, whose exponentials underflow in FP32
    (not in FP64).  The sums are kept as a running log-sum-exp, so the weights
    still match the oracle's FP64 ones, unnormalised and normalised."""
    from beep_gb300 import build
    build.build()
    rng = np.random.default_rng(12)
    tn, lp, tl, wl, ic = generation(rng, 64, 200)
    tn[:8] += 12.0 * np.sqrt(np.diag(np.linalg.inv(ic)))
    for norm in (False, True):
        g = capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.0, normalise=norm)
        o = oracle_abcsmc_weights(tn, lp, tl, wl, ic, 1.0, normalise=norm)
        assert np.all(np.isfinite(o))
        np.testing.assert_allclose(g, o, rtol=1e-5)


@pytest.mark.gpu
def test_gpu_weights_finite_where_every_term_underflows():
    """A new particle 40 standard deviations from every previous one: its
    kernel sum underflows even in FP64 (the reference's weight is then
    infinite).  The normalised weights stay finite; checked against an FP64
    log-sum-exp."""
    from beep_gb300 import build
    build.build()
    rng = np.random.default_rng(12)
    tn, lp, tl, wl, ic = generation(rng, 64, 200)
    tn[:8] += 40.0 * np.sqrt(np.diag(np.linalg.inv(ic)))
    g = capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.0)
    assert np.all(np.isfinite(g)) and np.all(g >= 0)
    np.testing.assert_allclose(g, _logsumexp_weights(tn, lp, tl, wl, ic, 1.0), rtol=1e-5, atol=1e-300)


@pytest.mark.gpu
def test_gpu_weights_full_generation_size():
    """16384 new against 16384 previous particles (the ABC-SMC generation of
    150 areas x 4 ages), against the oracle's FP64 weights."""
    from beep_gb300 import build
    build.build()
    rng = np.random.default_rng(13)
    tn, lp, tl, wl, ic = generation(rng, 16384, 16384)
    g = capi.abcsmc_weights(tn, lp, tl, wl, ic, 1.3)
    o = oracle_abcsmc_weights(tn, lp, tl, wl, ic, 1.3)
    np.testing.assert_allclose(g, o, rtol=1e-5)


@pytest.mark.gpu
def test_gpu_weights_reject_zero_previous_weights():
    from beep_gb300 import build
    build.build()
    tn, lp, tl, wl, ic = generation(np.random.default_rng(14), 4, 8)
    with pytest.raises(capi.BeepError):
        capi.abcsmc_weights(tn, lp, tl, np.zeros_like(wl), ic, 1.3)
