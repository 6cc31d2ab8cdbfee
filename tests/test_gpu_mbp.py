"""MBP chains on the GPU (beep_mbp_*, plain FP64 form) against the reference's
own Mbp (golden fixtures) and the oracle restatement."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import MBP_FIXTURES, MBP_VARIANTS, load, mbp_case, tn_checksums
from oracle_lib import oracle_mbp

pytestmark = pytest.mark.gpu

L_RTOL = 1e-12


@pytest.fixture(scope="module")
def device():
    capi.check(capi.lib().beep_device_init(0))
    return 0


@pytest.mark.parametrize("name", MBP_FIXTURES)
@pytest.mark.parametrize("v", range(MBP_VARIANTS))
def test_mbp_matches_reference(device, name, v):
    b, m, tabs, seed = load(name)
    gi, gp, si, sp, iu, simu = mbp_case(b, v)
    p = f"mbp{v}."
    nc = len(gi)
    dm = capi.DeviceModel(m)
    ch = capi.MbpChains(dm, nc)
    L0 = ch.initialise(tabs, seed, group_of=gi, stream_of=si)
    np.testing.assert_allclose(L0, b[p + "L_init"], rtol=L_RTOL, atol=0)
    np.testing.assert_allclose(ch.state_likelihood(tabs, group_of=gi), b[p + "Li_init"], rtol=L_RTOL, atol=0)
    np.testing.assert_allclose(ch.state_likelihood(tabs, group_of=gp), b[p + "Li_fixed"], rtol=L_RTOL, atol=0)
    L1 = ch.propose(tabs, seed, group_of=gp, stream_of=sp, inf_update=iu, simu=simu)
    np.testing.assert_allclose(L1, b[p + "L_prop"], rtol=L_RTOL, atol=0)
    nt = b[p + "transnum_init"].shape[0]
    for k in range(nc):
        tn, _ = ch.read_state(k)                 # still the initial state
        assert np.array_equal(tn_checksums(tn), b[p + "checksum"][k, 0])
        if k < nt:
            assert np.array_equal(tn, b[p + "transnum_init"][k])
    ch.accept(np.ones(nc, np.uint8))              # swap_initial_propose_state
    for k in range(nc):
        tn, _ = ch.read_state(k)
        assert np.array_equal(tn_checksums(tn), b[p + "checksum"][k, 1])
        if k < nt:
            assert np.array_equal(tn, b[p + "transnum_prop"][k])
    al = [capi.mbp_acceptance(False, 1.0, 0.0, -2 * L1[k], -2 * L0[k], b[p + "Pr_prop"][k], b[p + "Pr_init"][k])
          for k in range(nc)]
    np.testing.assert_allclose(al, b[p + "al"], rtol=1e-9, atol=1e-300)
    ch.close()
    dm.close()


def test_mbp_many_chains_match_oracle(device):
    """32 chains on the 10-area x 3-age workload, each kind of proposal, against
    the oracle; a partial acceptance leaves rejected chains on their initial state."""
    b, m, tabs, seed = load("c0_mbp")
    nc = 32
    ng = len(tabs)
    rng = np.random.default_rng(5)
    gi = rng.integers(0, ng, nc)
    gp = rng.integers(0, ng, nc)
    si = np.arange(nc, dtype=np.uint32) + 7000
    sp = np.arange(nc, dtype=np.uint32) + 9000
    simu = (rng.random((nc, m.ndivision, m.narea)) < 0.1).astype(np.uint8)
    dm = capi.DeviceModel(m)
    for iu, sm in ((capi.INF_DIF_UPDATE, None), (capi.INF_UPDATE, None), (capi.INF_DIF_UPDATE, simu)):
        o = oracle_mbp(m, tabs, gi, gp, seed, si, sp, iu, sm, want_tn=True)
        ch = capi.MbpChains(dm, nc)
        np.testing.assert_allclose(ch.initialise(tabs, seed, group_of=gi, stream_of=si), o["L_init"], rtol=L_RTOL)
        np.testing.assert_allclose(ch.state_likelihood(tabs, group_of=gp), o["Li_fixed"], rtol=L_RTOL)
        Lp = ch.propose(tabs, seed, group_of=gp, stream_of=sp, inf_update=iu, simu=sm)
        np.testing.assert_allclose(Lp, o["L_prop"], rtol=L_RTOL)
        acc = (np.arange(nc) % 3 == 0).astype(np.uint8)
        ch.accept(acc)
        for k in range(0, nc, 5):
            tn, _ = ch.read_state(k)
            assert np.array_equal(tn, o["tn_prop"][k] if acc[k] else o["tn_init"][k])
        ch.close()
    dm.close()


def test_mbp_errors(device):
    b, m, tabs, seed = load("tiny_mbp")
    dm = capi.DeviceModel(m)
    ch = capi.MbpChains(dm, 2)
    with pytest.raises(capi.BeepError) as e:
        ch.propose(tabs, seed)
    assert e.value.status == 1                    # BEEP_BAD_INPUT: not initialised
    with pytest.raises(capi.BeepError):
        capi.MbpChains(dm, 2, form=9)
    with pytest.raises(capi.BeepError):
        ch.propose(tabs, seed, inf_update=7)
    ch.close()
    dm.close()


def test_initialise_from_particle_restores_the_state(device):
    """beep_mbp_set_state (State::initialise_from_particle) from the counts of
    simulated chains rebuilds the same means bit for bit and the same
    likelihoods, and the next proposal from the rebuilt state is identical."""
    b, m, tabs, seed = load("c0_mbp")
    nc = 6
    gi = np.arange(nc) % len(tabs)
    dm = capi.DeviceModel(m)
    a = capi.MbpChains(dm, nc)
    L0 = a.initialise(tabs, seed, group_of=gi, stream_of=np.arange(nc) + 300)
    states = [a.read_state(k) for k in range(nc)]
    tn = np.stack([s_[0] for s_ in states])
    c = capi.MbpChains(dm, nc)
    Lc = c.set_state(tabs, tn, group_of=gi)
    np.testing.assert_allclose(Lc, L0, rtol=1e-12)
    for k in range(nc):
        tn2, mean2 = c.read_state(k)
        assert np.array_equal(tn2, states[k][0])
        assert np.array_equal(mean2, states[k][1])
    np.testing.assert_array_equal(c.state_likelihood(tabs, group_of=gi), a.state_likelihood(tabs, group_of=gi))
    gp = (gi + 1) % len(tabs)
    for ch in (a, c):
        ch.propose(tabs, seed, group_of=gp, stream_of=np.arange(nc) + 900, inf_update=capi.INF_DIF_UPDATE)
        ch.accept(np.ones(nc, np.uint8))
    for k in range(nc):
        assert np.array_equal(a.read_state(k)[0], c.read_state(k)[0])
    a.close()
    c.close()
    dm.close()


def test_fast_chains_follow_plain_chains(device):
    """Fast-form chains (FP32 means, same keyed streams, FP32 binomial
    inversion) follow the plain FP64 chains: most initial states and coupled
    proposals are identical, with log-likelihoods within 1e-6 and state
    likelihoods within 1e-5 where they are."""
    b, m, tabs, seed = load("c0_mbp")
    nc = 32
    gi = np.arange(nc) % len(tabs)
    gp = (gi + 3) % len(tabs)
    dm = capi.DeviceModel(m)
    res = {}
    for form in (capi.FORM_PLAIN_FP64, capi.FORM_FAST):
        ch = capi.MbpChains(dm, nc, form=form)
        L0 = ch.initialise(tabs, seed, group_of=gi, stream_of=np.arange(nc) + 100)
        tn0 = np.stack([ch.read_state(k)[0] for k in range(nc)])
        Li = ch.state_likelihood(tabs, group_of=gp)
        L1 = ch.propose(tabs, seed, group_of=gp, stream_of=np.arange(nc) + 400, inf_update=capi.INF_DIF_UPDATE)
        ch.accept(np.ones(nc, np.uint8))
        tn1 = np.stack([ch.read_state(k)[0] for k in range(nc)])
        res[form] = (L0, tn0, Li, L1, tn1)
        ch.close()
    (pL0, ptn0, pLi, pL1, ptn1), (fL0, ftn0, fLi, fL1, ftn1) = res[capi.FORM_PLAIN_FP64], res[capi.FORM_FAST]
    same0 = np.array([np.array_equal(ptn0[k], ftn0[k]) for k in range(nc)])
    assert same0.mean() >= 0.6, same0.mean()
    np.testing.assert_allclose(fL0[same0], pL0[same0], rtol=1e-6)
    np.testing.assert_allclose(fLi[same0], pLi[same0], rtol=1e-5)
    same1 = same0 & np.array([np.array_equal(ptn1[k], ftn1[k]) for k in range(nc)])
    assert same1.mean() >= 0.4, same1.mean()
    np.testing.assert_allclose(fL1[same1], pL1[same1], rtol=1e-6)
    dm.close()


def test_fast_chains_state_round_trip(device):
    b, m, tabs, seed = load("tiny_mbp")
    nc = 4
    gi = np.arange(nc) * 2
    dm = capi.DeviceModel(m)
    a = capi.MbpChains(dm, nc, form=capi.FORM_FAST)
    L0 = a.initialise(tabs, seed, group_of=gi, stream_of=np.arange(nc) + 7)
    st = [a.read_state(k) for k in range(nc)]
    c = capi.MbpChains(dm, nc, form=capi.FORM_FAST)
    Lc = c.set_state(tabs, np.stack([x[0] for x in st]), group_of=gi)
    np.testing.assert_allclose(Lc, L0, rtol=1e-6)
    for k in range(nc):
        tn, mean = c.read_state(k)
        assert np.array_equal(tn, st[k][0])
        np.testing.assert_allclose(mean, st[k][1], rtol=1e-6)
    a.close()
    c.close()
    dm.close()


@pytest.fixture
def ctas_option(device):
    yield capi.set_option
    capi.set_option("fast_ctas_per_sm", 0)


def test_fast_chains_several_per_sm_follow_plain_chains(ctas_option):
    """Fast chains in 320-thread CTAs, four per SM, on a model of 70 areas x 4
    ages (280 columns, 30 days): the same arithmetic per column as one
    640-thread CTA per SM (identical states, log-likelihoods within 1e-6), and
    the initial states and coupled proposals follow the plain FP64 chains."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260205, narea=70, nage=4, days=30, name="mbp70")
    w.obs_kind = "hosp_pop"
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    nc = 24
    go = np.zeros(nc, np.int32)
    dm = capi.DeviceModel(m)
    res = {}
    for form, k in ((capi.FORM_PLAIN_FP64, 0), (capi.FORM_FAST, 1), (capi.FORM_FAST, 4)):
        ctas_option("fast_ctas_per_sm", k)
        ch = capi.MbpChains(dm, nc, form=form)
        L0 = ch.initialise([t], 17, group_of=go, stream_of=np.arange(nc) + 100)
        tn0 = np.stack([ch.read_state(i)[0] for i in range(nc)])
        L1 = ch.propose([t], 18, group_of=go, stream_of=np.arange(nc) + 400, inf_update=capi.INF_DIF_UPDATE)
        ch.accept(np.ones(nc, np.uint8))
        tn1 = np.stack([ch.read_state(i)[0] for i in range(nc)])
        if form == capi.FORM_FAST:
            assert ch.ctas_per_sm() == k, (k, ch.ctas_per_sm())
        res[(form, k)] = (L0, tn0, L1, tn1)
        ch.close()
    # same draws; the log-likelihood's per-thread partial sums group differently
    r1, r4 = res[(capi.FORM_FAST, 1)], res[(capi.FORM_FAST, 4)]
    assert np.array_equal(r1[1], r4[1]) and np.array_equal(r1[3], r4[3])
    np.testing.assert_allclose(r4[0], r1[0], rtol=1e-6)
    np.testing.assert_allclose(r4[2], r1[2], rtol=1e-6)
    pL0, ptn0, pL1, ptn1 = res[(capi.FORM_PLAIN_FP64, 0)]
    fL0, ftn0, fL1, ftn1 = res[(capi.FORM_FAST, 4)]
    same0 = np.array([np.array_equal(ptn0[i], ftn0[i]) for i in range(nc)])
    assert same0.mean() >= 0.5, same0.mean()
    np.testing.assert_allclose(fL0[same0], pL0[same0], rtol=1e-6)
    same1 = same0 & np.array([np.array_equal(ptn1[i], ftn1[i]) for i in range(nc)])
    assert same1.mean() >= 0.3, same1.mean()
    np.testing.assert_allclose(fL1[same1], pL1[same1], rtol=1e-6)
    dm.close()
