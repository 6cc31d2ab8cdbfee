"""Log-prior and bounds (beep_log_prior) against the reference's own
Model::prior / Model::inbounds (src/model.cc:1590-1706, 2625-2669), recorded by
the reference harness for parameter rows around the workloads' values and for
probe rows outside the bounds (each parameter in turn below or above its
uniform range, or scaled by 1.1).  The specification comes through the
binding (beep_gb300/binding, PriorPack).  Host code: no GPU."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import load


@pytest.mark.parametrize("name", ["prior_spec", "c0_mbp"])
def test_log_prior_and_bounds_match_reference(name):
    from beep_gb300 import build
    build.build()
    b, m, tabs, seed = load(name)
    pr = capi.Priors(b)
    lp, ib = pr.evaluate(b["prior.theta"])
    ref_ib = b["prior.inbounds"].astype(bool)
    assert ref_ib.any() and (~ref_ib).any()
    assert np.array_equal(ib, ref_ib)
    np.testing.assert_allclose(lp[ib], b["prior.logprior"][ref_ib], rtol=1e-12, atol=1e-12)
    assert np.all(np.isneginf(lp[~ib]))


def test_spline_smoothing_term_is_used():
    """The prior fixture smooths R(t) (log-normal smoothing): dropping the
    smoothing terms changes the log-prior by the reference's spline_prior."""
    b, m, tabs, seed = load("prior_spec")
    pr = capi.Priors(b)
    assert pr.st.nsmooth > 0
    full, _ = pr.evaluate(b["prior.theta"][:1])
    nosm = dict(b)
    nosm["prior.smooth_kind"] = np.zeros(0, np.int32)
    part, _ = capi.Priors(nosm).evaluate(b["prior.theta"][:1])
    assert full[0] != part[0]


def test_mbp_acceptance_priors_match_reference():
    """The MBP fixture's Pr of every chain's start and proposal rows (the
    reference's State::Pr, set through Model::prior) equals beep_log_prior."""
    b, m, tabs, seed = load("c0_mbp")
    pr = capi.Priors(b)
    nc = int(b["mbp.nchain"][0])
    rows = np.stack([b[f"g{k}.theta"] for k in range(2 * nc)])
    lp, ib = pr.evaluate(rows)
    assert ib.all()
    np.testing.assert_allclose(lp[0::2], b["mbp0.Pr_init"], rtol=1e-12)
    np.testing.assert_allclose(lp[1::2], b["mbp0.Pr_prop"], rtol=1e-12)
