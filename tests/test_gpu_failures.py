"""Failure statuses that the kernels raise from arithmetic, made to fire:

* BEEP_COUNT_OVERFLOW: a transition mean above 1e9 (the int32 counts could
  not hold the draw) -- here from beta rows scaled up on the host;
* BEEP_TIMEOUT from the samplers: a rejection sampler that runs out of
  iterations -- here with the library's iteration limit lowered to one
  iteration (option sampler_iteration_limit), so that some of the thousands
  of PTRS / BTRS draws of a run reject on their only try.

Both are plain arithmetic on the device: nothing waits, nothing faults, and
the model stays usable afterwards (the next batch gives the usual result)."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import load

pytestmark = pytest.mark.gpu
L_RTOL = 1e-12
FORMS = [capi.FORM_PLAIN_FP64, capi.FORM_FAST]


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    yield capi.lib()
    capi.set_option("sampler_iteration_limit", 0)


@pytest.mark.parametrize("form", FORMS)
def test_count_overflow_is_reported(built, form):
    b, m, tabs, seed = load("c0_sim")
    dm = capi.DeviceModel(m)
    big = capi.Tables({k: (v * 1e15 if k == "g0.beta_rows" else v) for k, v in b.items()}, "g0.")
    with pytest.raises(capi.BeepError) as e:
        dm.simulate(capi.Batch(m, [big], 4, seed, form=form))
    assert e.value.status == 7, e.value
    ok = dm.simulate(capi.Batch(m, tabs, 4, seed))
    np.testing.assert_allclose(ok.L, b["g0.L"][:4], rtol=L_RTOL)
    dm.close()


@pytest.mark.parametrize("form", FORMS)
def test_sampler_iteration_limit_is_reported(built, form):
    b, m, tabs, seed = load("c0_sim")
    dm = capi.DeviceModel(m)
    ref = dm.simulate(capi.Batch(m, tabs, 16, seed, form=form))
    capi.set_option("sampler_iteration_limit", 1)
    try:
        with pytest.raises(capi.BeepError) as e:
            dm.simulate(capi.Batch(m, tabs, 16, seed, form=form))
        assert e.value.status == 4, e.value
    finally:
        capi.set_option("sampler_iteration_limit", 0)
    again = dm.simulate(capi.Batch(m, tabs, 16, seed, form=form))
    assert np.array_equal(again.L, ref.L)
    dm.close()


def test_mbp_thinning_iteration_limit_is_reported(built):
    """The coupled MBP proposal's binomial thinning (BTRS) under the same limit."""
    b, m, tabs, seed = load("c0_mbp")
    dm = capi.DeviceModel(m)
    ch = capi.MbpChains(dm, 16)
    ch.initialise(tabs[:1], seed, group_of=np.zeros(16, np.int32))
    # a proposal whose infection means are a little below the current ones: the coupled
    # infection counts are thinned with p near 0.9 (q = 0.1), by BTRS wherever n q >= 10
    # (a steeper cut would let the proposal fall behind, p drop and inversion take over)
    low = capi.Tables({k: (v * 0.9 if k == "g0.beta_rows" else v) for k, v in b.items()}, "g0.")
    capi.set_option("sampler_iteration_limit", 1)
    try:
        with pytest.raises(capi.BeepError) as e:
            ch.propose([low], seed + 1, group_of=np.zeros(16, np.int32))
        assert e.value.status == 4, e.value
    finally:
        capi.set_option("sampler_iteration_limit", 0)
    ch.close()
    dm.close()
