"""CUDA-graph replay of a batch step and the fast form's autotuner."""
import numpy as np
import pytest

from beep_gb300 import capi, model_builder as mb, synth
from golden_util import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    return capi.lib()


@pytest.mark.parametrize("form", [capi.FORM_PLAIN_FP64, capi.FORM_FAST])
def test_graph_replay_equals_plain_launches(built, form):
    b, m, tabs, seed = load("c0_sim")
    dm = capi.DeviceModel(m)
    P = 96
    ref = dm.simulate(capi.Batch(m, tabs, P, seed, want_pop=True, form=form))
    bt = capi.Batch(m, tabs, P, seed, want_pop=True, form=form)
    db = capi.DeviceBatch(dm, bt)
    for _ in range(3):                       # capture, then replays
        bt.L[:] = 0
        bt.pop[:] = 0
        db.run_graph()
        assert np.array_equal(bt.L, ref.L) and np.array_equal(bt.pop, ref.pop)
    db.close()
    dm.close()


def test_graph_replay_follows_new_inputs(built):
    """The staged inputs are re-packed before every replay: new parameter
    tables of the same size change the results like a fresh batch would."""
    w = synth.abc_smc_large(narea=30, nage=2, days=40)
    m = capi.Model(mb.model_arrays(w))
    rng = np.random.default_rng(3)
    P = 64
    R0, si, gi = synth.abc_smc_priors(rng, P)
    t1 = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
    R0b, sib, gib = synth.abc_smc_priors(rng, P)
    t2 = [capi.Tables(t) for t in mb.param_tables_batch(w, R0b, sib, gib)]
    dm = capi.DeviceModel(m)
    bt = capi.Batch(m, t1, P, 5, group_of=np.arange(P), form=capi.FORM_FAST)
    db = capi.DeviceBatch(dm, bt)
    db.run_graph()
    L1 = bt.L.copy()
    for k in range(P):                        # swap the parameter sets in place
        bt.groups[k] = t2[k].st
    bt.tables = t2
    db.run_graph()
    ref = dm.simulate(capi.Batch(m, t2, P, 5, group_of=np.arange(P), form=capi.FORM_FAST))
    assert np.array_equal(bt.L, ref.L) and not np.array_equal(bt.L, L1)
    db.close()
    dm.close()


def test_autotuner_records_a_supported_path(built):
    w = synth.seir_hd_small(seed=20260300, narea=120, nage=3, days=40, name="tune")
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    dm = capi.DeviceModel(m)
    bt = capi.Batch(m, [t], 400, 1, form=capi.FORM_FAST)
    chosen = dm.autotune(bt)
    assert chosen in (capi.FOI_SIMT, capi.FOI_TENSOR)
    db = capi.DeviceBatch(dm, bt)
    assert db.foi_path() == chosen            # later batches of the model use the choice
    assert db.ctas_per_sm() >= 1 and (chosen == capi.FOI_SIMT or db.ctas_per_sm() == 1)
    r = db.run()
    assert np.isfinite(r.L).all()
    db.close()
    dm.close()
