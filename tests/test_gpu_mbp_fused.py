"""MBP chains of several models in one persistent launch
(beep_mbp_propose_fused) against each set's own launch (beep_mbp_propose):
the chains of the uneven-size chain workload (20x2, 80x4, 200x6 and 350x10
areas x ages, 200 days at dt 0.5, weekly hospital populations) draw the same
proposals, with log-likelihoods within the fast form's 1e-6."""
import numpy as np
import pytest

from beep_gb300 import capi, model_builder as mb, synth

pytestmark = pytest.mark.gpu

NCHAIN = 8


def chain_model(A, G, rng):
    """One model of the workload, observed data from one fast simulation."""
    w = synth.mbp_chain_model(A, G)
    arr0 = mb.model_arrays(w)
    m0 = capi.Model(arr0)
    dm0 = capi.DeviceModel(m0)
    truth = dm0.simulate(capi.Batch(m0, [capi.Tables(mb.param_tables(w))], 1, 11 + A, want_transnum=True,
                                    want_pop_traj=True, want_L=False, form=capi.FORM_FAST))
    dm0.close()
    y, sd = mb.observed_from_trajectory(arr0, truth.transnum[0], truth.pop_traj[0], rng)
    arr = dict(arr0)
    arr["obs_value"], arr["obs_sd"] = y, sd
    return w, capi.Model(arr)


def tables_for(w, rng, n):
    th = np.stack([rng.uniform(2.2, 2.8, n), rng.uniform(3.6, 4.4, n), rng.uniform(4.5, 5.5, n)], 1)
    return [capi.Tables(t) for t in mb.param_tables_batch(w, th[:, 0], th[:, 1], th[:, 2])]


@pytest.fixture(scope="module")
def chains():
    capi.check(capi.lib().beep_device_init(0))
    rng = np.random.default_rng(20260411)
    out = []
    for (A, G) in synth.MBP_SIZES:
        w, m = chain_model(A, G, rng)
        dm = capi.DeviceModel(m)
        t0 = tables_for(w, rng, NCHAIN)
        sets = []
        for _ in range(2):      # separate launches / fused launch, same initial states
            ch = capi.MbpChains(dm, NCHAIN, form=capi.FORM_FAST)
            ch.initialise(t0, 5, group_of=np.arange(NCHAIN), stream_of=np.arange(NCHAIN))
            sets.append(ch)
        out.append(dict(w=w, m=m, dm=dm, sep=sets[0], fus=sets[1], rng=rng))
    yield out
    for x in out:
        x["sep"].close()
        x["fus"].close()
        x["dm"].close()


def states(ch):
    return np.stack([ch.read_state(k)[0] for k in range(ch.nchain)])


def test_fused_launch_draws_each_sets_proposals(chains):
    """Two sweeps: every set proposed in its own launch and all four sets in one
    fused launch from the same states give identical proposed counts; L within
    1e-6 (sets whose own launch runs 640 threads per chain: identical)."""
    for sweep in range(2):
        reqs = []
        for i, x in enumerate(chains):
            reqs.append(dict(tables=tables_for(x["w"], x["rng"], NCHAIN), seed=77 + sweep,
                             group_of=np.arange(NCHAIN), stream_of=np.arange(NCHAIN) + (sweep + 1) * NCHAIN,
                             inf_update=capi.INF_DIF_UPDATE))
        L_sep = [x["sep"].propose(**r) for x, r in zip(chains, reqs)]
        # sets passed smallest first: the launch orders them by cost itself
        L_fus = capi.MbpChains.propose_fused([x["fus"] for x in chains], reqs)
        for x, ls, lf in zip(chains, L_sep, L_fus):
            assert np.all(np.isfinite(lf))
            np.testing.assert_allclose(lf, ls, rtol=1e-6)
            acc = (np.arange(NCHAIN) + sweep) % 2 == 0      # accept half, the other half keeps its state
            x["sep"].accept(acc.astype(np.uint8))
            x["fus"].accept(acc.astype(np.uint8))
            assert np.array_equal(states(x["sep"]), states(x["fus"])), f"{x['m'].narea}x{x['m'].nage}"
        big = chains[-1]
        assert big["m"].narea * big["m"].ndemocatpos > 256          # 640 threads alone too: same L bits
        assert np.array_equal(L_fus[-1], L_sep[-1])


def test_fused_launch_rejects_bad_sets(chains):
    x = chains[0]
    r = dict(tables=tables_for(x["w"], x["rng"], NCHAIN), seed=1, group_of=np.arange(NCHAIN))
    with pytest.raises(capi.BeepError) as e:
        capi.MbpChains.propose_fused([x["fus"], x["fus"]], [r, r])
    assert e.value.status == 1   # BEEP_BAD_INPUT
    plain = capi.MbpChains(x["dm"], NCHAIN, form=capi.FORM_PLAIN_FP64)
    plain.initialise(r["tables"], 3, group_of=np.arange(NCHAIN))
    with pytest.raises(capi.BeepError) as e:
        capi.MbpChains.propose_fused([x["fus"], plain], [r, r])
    assert e.value.status == 1   # BEEP_BAD_INPUT
    fresh = capi.MbpChains(x["dm"], NCHAIN, form=capi.FORM_FAST)   # not initialised
    with pytest.raises(capi.BeepError) as e:
        capi.MbpChains.propose_fused([fresh], [r])
    assert e.value.status == 1   # BEEP_BAD_INPUT
    plain.close()
    fresh.close()
