"""Demographic changes (State::democat_change_pop_adjust, src/state.cc:339-376):
before every step the populations move between the values of a demographic
classification so that their shares follow the change's per-step fractions.
Populations stop being integers, so such models run the plain FP64 form with
FP64 populations.

* the plain form against the oracle on a 60-area x 4-age model with two
  changes (every area; two areas), 48 particles over 200 steps: transition
  counts, FP64 populations and their trajectories bit-exact, L to 1e-12;
* the same in two sections, populations carried in FP64 (pop_in_f64);
* the reference's own fixtures (whole run, filter sections, MBP chains) run
  through the parity, filter and MBP tests (golden_util's fixture lists);
* the fast form, fast MBP chains, the allocation-free entry point and the
  int32 population fields refuse such a model, and the FP64 fields refuse a
  model without changes;
* a serving request of such a model gives what it gives alone."""
import ctypes as C

import numpy as np
import pytest

from beep_gb300 import capi, model_builder as mb, synth
from golden_util import load
from oracle_lib import oracle_simulate

pytestmark = pytest.mark.gpu
L_RTOL = 1e-12


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    return capi.lib()


@pytest.fixture(scope="module")
def model60():
    w = synth.seir_hd_democat(seed=20260111, narea=60, nage=4, days=100, name="democat60")
    arr = mb.model_arrays(w)
    m = capi.Model(arr)
    assert m.pop64 and m.ndemocat_change == 2
    rng = np.random.default_rng(3)
    tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, rng.uniform(1.5, 3.0, 3), rng.uniform(3, 5, 3),
                                                          rng.uniform(4, 6, 3))]
    return w, m, tabs


def test_plain_form_matches_oracle(built, model60):
    w, m, tabs, = model60
    P = 48
    go = np.arange(P) % len(tabs)
    dm = capi.DeviceModel(m)
    g = dm.simulate(capi.Batch(m, tabs, P, 77, group_of=go, want_transnum=True, want_pop=True, want_pop_traj=True))
    dm.close()
    o = oracle_simulate(m, capi.Batch(m, tabs, P, 77, group_of=go, want_transnum=True, want_pop=True,
                                      want_pop_traj=True))
    assert g.pop.dtype == np.float64
    assert np.mean(g.pop != np.round(g.pop)) > 0.5          # the populations are fractional
    assert g.transnum.sum() > 0
    assert np.array_equal(g.transnum, o.transnum)
    assert np.array_equal(g.pop_traj, o.pop_traj)
    assert np.array_equal(g.pop, o.pop)
    np.testing.assert_allclose(g.L, o.L, rtol=L_RTOL, atol=0)


def test_sections_carry_fp64_populations(built, model60):
    w, m, tabs = model60
    P, S = 16, m.ndivision
    dm = capi.DeviceModel(m)
    res = []
    for run in (dm.simulate, lambda bt: oracle_simulate(m, bt)):
        a = run(capi.Batch(m, tabs, P, 5, ti=0, tf=S // 2, want_transnum=True, want_pop=True))
        b = run(capi.Batch(m, tabs, P, 5, ti=S // 2, tf=S, pop_in=a.pop, want_transnum=True, want_pop=True))
        res.append((a, b))
    dm.close()
    (ga, gb), (oa, ob) = res
    for x, y in ((ga, oa), (gb, ob)):
        assert np.array_equal(x.transnum, y.transnum)
        assert np.array_equal(x.pop, y.pop)
        np.testing.assert_allclose(x.L, y.L, rtol=L_RTOL, atol=1e-12)


def test_other_forms_and_fields_refuse(built):
    b, m, tabs, seed = load("democat_sim")
    dm = capi.DeviceModel(m)
    with pytest.raises(capi.BeepError) as e:
        dm.simulate(capi.Batch(m, tabs, 4, seed, form=capi.FORM_FAST))
    assert e.value.status == 1
    with pytest.raises(capi.BeepError) as e:
        capi.MbpChains(dm, 4, form=capi.FORM_FAST)
    assert e.value.status == 1
    # int32 population fields on a model with changes
    bt = capi.Batch(m, tabs, 4, seed, want_pop=True)
    ipop = np.zeros((4, m.narea, m.ncomp, m.ndemocatpos), np.int32)
    bt.st.pop_out = ipop.ctypes.data_as(C.POINTER(C.c_int32))
    bt.st.pop_out_f64 = None
    with pytest.raises(capi.BeepError):
        dm.simulate(bt)
    # the allocation-free entry point (checked before any table pointer is read)
    st = capi.ParamTables()
    L = C.c_double(0)
    r = capi.lib().beep_simulate_plain_noalloc(dm.h, C.byref(st), 1, seed, 0, m.ndivision, None, C.byref(L), None,
                                               None)
    assert r == 1 and b"demographic" in capi.lib().beep_last_error()
    dm.close()
    # FP64 population fields on a model without changes
    b2, m2, t2, s2 = load("tiny_sim")
    dm2 = capi.DeviceModel(m2)
    bt2 = capi.Batch(m2, t2, 2, s2)
    fp = np.zeros((2, m2.narea, m2.ncomp, m2.ndemocatpos))
    bt2.st.pop_out_f64 = fp.ctypes.data_as(C.POINTER(C.c_double))
    with pytest.raises(capi.BeepError):
        dm2.simulate(bt2)
    dm2.close()


def test_serving_request_same_as_alone(built):
    b, m, tabs, seed = load("democat_sim")
    dm = capi.DeviceModel(m)
    alone = dm.simulate(capi.Batch(m, tabs, 6, seed, want_pop=True, want_transnum=True))
    dm.close()
    srv = capi.Server(4 << 30, 2)
    bts = [capi.Batch(m, tabs, 6, seed, want_pop=True, want_transnum=True) for _ in range(2)]
    ts = [srv.submit(m, bt, capi.REQ_LIKELIHOOD) for bt in bts]
    for t, bt in zip(ts, bts):
        srv.wait(t, 120.0)
        assert np.array_equal(bt.pop, alone.pop)
        assert np.array_equal(bt.transnum, alone.transnum)
        assert np.array_equal(bt.L, alone.L)
    srv.close()
