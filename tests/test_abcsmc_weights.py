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
