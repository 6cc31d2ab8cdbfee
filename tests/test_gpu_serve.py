"""Serving loop (beep_server_*): requests of uneven sizes admitted by device
footprint and run concurrently give exactly the results they give alone."""
import numpy as np
import pytest

from beep_gb300 import capi, model_builder as mb, synth
from golden_util import load

pytestmark = pytest.mark.gpu


def synthetic(narea, nage, days, steps_per_day, seed):
    w = synth.seir_hd_small(seed=seed, narea=narea, nage=nage, days=days, steps_per_day=steps_per_day,
                            name=f"s{narea}x{nage}")
    m = capi.Model(mb.model_arrays(w))
    rng = np.random.default_rng(seed)
    n = 4
    tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, rng.uniform(1.5, 3.0, n), rng.uniform(3, 5, n),
                                                          rng.uniform(4, 6, n))]
    return m, tabs


def request_specs():
    """(kind, model, tables, batch kwargs) of a mixed stream."""
    specs = []
    b, m, tabs, seed = load("tiny_sim")
    specs.append((capi.REQ_LIKELIHOOD, m, tabs, dict(nparticle=8, seed=seed)))
    b, m, tabs, seed = load("c0_sim")
    specs.append((capi.REQ_LIKELIHOOD, m, tabs, dict(nparticle=256, seed=11, form=capi.FORM_FAST)))
    specs.append((capi.REQ_SCENARIO, m, tabs, dict(nparticle=4, seed=12, want_L=False, want_transnum=True,
                                                    want_pop_traj=True)))
    half = m.ndivision // 2
    specs.append((capi.REQ_PREDICTION, m, tabs, dict(nparticle=16, seed=13, ti=half, want_pop=True,
                                                      form=capi.FORM_FAST, prediction_from=half)))
    m2, t2 = synthetic(60, 4, 60, 4, 20260400)
    specs.append((capi.REQ_LIKELIHOOD, m2, t2, dict(nparticle=600, seed=14, group_of=np.arange(600) % 4,
                                                     form=capi.FORM_FAST)))
    m3, t3 = synthetic(120, 6, 40, 2, 20260401)
    specs.append((capi.REQ_LIKELIHOOD, m3, t3, dict(nparticle=200, seed=15, group_of=np.arange(200) % 4,
                                                     form=capi.FORM_FAST, want_pop=True)))
    specs.append((capi.REQ_LIKELIHOOD, m3, t3, dict(nparticle=24, seed=16, group_of=np.arange(24) % 4)))
    return specs


def make_batch(dm, m, tabs, kw):
    kw = dict(kw)
    P = kw.pop("nparticle")
    seed = kw.pop("seed")
    frm = kw.pop("prediction_from", None)
    if frm is not None:
        # populations at step `frm` of a run from the start (PREDICTION continues them)
        pre = dm.simulate(capi.Batch(m, tabs, P, seed + 1000, tf=frm, want_L=False, want_pop=True,
                                     group_of=kw.get("group_of")))
        kw["pop_in"] = pre.pop
    return capi.Batch(m, tabs, P, seed, **kw)


def outputs(bt):
    return {k: getattr(bt, k) for k in ("L", "pop", "transnum", "pop_traj") if getattr(bt, k) is not None}


@pytest.fixture(scope="module")
def alone():
    """Every request run alone through beep_simulate."""
    res = []
    for kind, m, tabs, kw in request_specs():
        dm = capi.DeviceModel(m)
        bt = make_batch(dm, m, tabs, kw)
        res.append((kind, m, tabs, bt, outputs(dm.simulate(bt))))
        dm.close()
    return res


def resubmit(srv, alone_runs):
    tickets, batches = [], []
    for kind, m, tabs, bt, _ in alone_runs:
        b2 = capi.Batch(m, tabs, bt.st.nparticle, bt.st.seed, ti=bt.st.ti, tf=bt.st.tf,
                        group_of=bt.group_of, pop_in=bt.pop_in, want_L=bt.L is not None, want_pop=bt.pop is not None,
                        want_transnum=bt.transnum is not None, want_pop_traj=bt.pop_traj is not None, form=bt.st.form)
        batches.append(b2)
        tickets.append(srv.submit(m, b2, kind))
    return tickets, batches


@pytest.mark.parametrize("budget,inflight", [(8 << 30, 4), (1, 4), (8 << 30, 1)])
def test_results_same_alone_and_in_the_mix(alone, budget, inflight):
    srv = capi.Server(budget, inflight)
    tickets, batches = resubmit(srv, alone)
    for t, b2, (_, _, _, _, ref) in zip(tickets, batches, alone):
        srv.wait(t, 120.0)
        got = outputs(b2)
        assert got.keys() == ref.keys()
        for k in ref:
            assert np.array_equal(got[k], ref[k]), k      # bit-identical, whatever ran beside it
    st = [srv.stats(t) for t in tickets]
    assert all(s["state"] == 2 and s["status"] == 0 for s in st)
    order = sorted(st, key=lambda s: s["admit_s"])
    if budget == 1 or inflight == 1:
        # one request at a time: each is admitted after the previous finished
        for a, b in zip(order, order[1:]):
            assert b["admit_s"] >= a["done_s"] - 1e-6
    for t in tickets:
        srv.release(t)
    srv.close()


def test_concurrent_requests_overlap_on_the_device():
    m, tabs = synthetic(100, 4, 120, 4, 20260402)
    srv = capi.Server(16 << 30, 4)
    bs = [capi.Batch(m, tabs, 3000, 100 + k, group_of=np.arange(3000) % 4, form=capi.FORM_FAST) for k in range(4)]
    ts = [srv.submit(m, b, capi.REQ_LIKELIHOOD) for b in bs]
    for t in ts:
        srv.wait(t, 120.0)
    iv = sorted((srv.stats(t)["gpu_start_s"], srv.stats(t)["gpu_end_s"]) for t in ts)
    assert any(iv[k + 1][0] < iv[k][1] for k in range(len(iv) - 1)), iv
    srv.close()


def test_bad_requests():
    b, m, tabs, seed = load("tiny_sim")
    srv = capi.Server(1 << 30, 2)
    bt = capi.Batch(m, tabs, 4, seed, want_L=False, want_pop=True)
    with pytest.raises(capi.BeepError):
        srv.submit(m, bt, capi.REQ_LIKELIHOOD)          # a likelihood request without L_out
    with pytest.raises(capi.BeepError):
        srv.submit(m, bt, 7)                            # unknown kind
    bad = capi.Batch(m, tabs, 4, seed, group_of=[0, 5, 0, 0])
    t = srv.submit(m, bad, capi.REQ_LIKELIHOOD)        # rejected when admitted
    with pytest.raises(capi.BeepError) as e:
        srv.wait(t, 60.0)
    assert e.value.status == 1
    ok = capi.Batch(m, tabs, 4, seed)
    t2 = srv.submit(m, ok, capi.REQ_LIKELIHOOD)        # the server keeps serving
    srv.wait(t2, 60.0)
    np.testing.assert_allclose(ok.L, b["g0.L"][:4], rtol=1e-12)
    srv.close()


def test_particle_filter_requests_alone_and_in_the_mix():
    """Particle-filter requests (states resident on the device between
    sections) give the estimate, section terms, ancestors and lineage they give
    through beep_pf_loglik alone, while simulation requests run beside them."""
    b, m, tabs, seed = load("c0_pf")
    dm = capi.DeviceModel(m)
    cases = [(128, seed + 1, capi.FORM_PLAIN_FP64), (256, seed + 2, capi.FORM_FAST), (64, seed + 3, capi.FORM_PLAIN_FP64)]
    alone = [dm.pf_loglik(tabs[0], N, sd, 5, 1.0, m.sections, form=f, lineage=True) for N, sd, f in cases]
    dm.close()
    srv = capi.Server(8 << 30, 4)
    ts = [srv.submit_pf(m, tabs[0], N, sd, 5, 1.0, m.sections, form=f, lineage=True) for N, sd, f in cases]
    mw, tw = synthetic(60, 4, 60, 4, 20260410)
    sims = [capi.Batch(mw, tw, 500, 30 + k, group_of=np.arange(500) % 4, form=capi.FORM_FAST) for k in range(3)]
    tsim = [srv.submit(mw, bt, capi.REQ_LIKELIHOOD) for bt in sims]
    for t, ref in zip(ts, alone):
        out = srv.wait(t, 120.0)
        assert out["loglik"][0] == ref[0]
        assert np.array_equal(out["loglik_section"], ref[1])
        assert np.array_equal(out["ancestors"], ref[3])
        assert np.array_equal(out["lineage"], ref[4])
    for t in tsim:
        srv.wait(t, 120.0)
    srv.close()


@pytest.mark.parametrize("form", [capi.FORM_PLAIN_FP64, capi.FORM_FAST])
def test_requests_of_one_model_are_packed_into_one_batch(form):
    """Queued requests of the same model, form, step range and outputs run as
    one batch: their parameter sets, streams and seeds are concatenated, and
    each request gets what it gets alone -- the same counts and populations,
    and L bit for bit in the plain form (within the fast form's 1e-6 where the
    pack's size gives the fast kernel another layout)."""
    m, tabs = synthetic(100, 4, 60, 4, 20260403)
    rng = np.random.default_rng(7)
    sizes = [40, 300, 17, 900, 64]
    specs = []
    for k, P in enumerate(sizes):
        t = [tabs[j] for j in rng.permutation(len(tabs))[:2]]
        specs.append((t, P, 500 + 31 * k, rng.integers(0, 2, P)))
    dm = capi.DeviceModel(m)
    alone = [dm.simulate(capi.Batch(m, t, P, sd, group_of=go, want_pop=True, form=form)) for t, P, sd, go in specs]
    dm.close()
    srv = capi.Server(16 << 30, 1)
    bs = [capi.Batch(m, t, P, sd, group_of=go, want_pop=True, form=form) for t, P, sd, go in specs]
    ts = [srv.submit(m, b, capi.REQ_LIKELIHOOD) for b in bs]
    for t in ts:
        srv.wait(t, 120.0)
    st = [srv.stats(t) for t in ts]
    spans = [(s["gpu_start_s"], s["gpu_end_s"]) for s in st]
    assert len(set(spans)) < len(spans), spans          # at least two requests shared one batch
    for b, ref in zip(bs, alone):
        assert np.array_equal(b.pop, ref.pop)
        if form == capi.FORM_PLAIN_FP64:
            assert np.array_equal(b.L, ref.L)
        else:
            np.testing.assert_allclose(b.L, ref.L, rtol=1e-6)
    srv.close()
