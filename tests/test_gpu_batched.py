"""Fast form in the step-synchronous layout (sim_batched.cu): every particle
advances one step at a time and the area-mixing contraction of the force of
infection is one tensor-core product over the whole batch per step
([P*NS*G x A] . [A x A], split BF16 pieces, FP32 accumulation).

Same keyed variate streams and the same per-column FP32 arithmetic as the
other fast-form layouts, so particles follow the FP64 form's trajectories
except where an FP32 comparison lands on the other side of a near tie; the
log-likelihood of an identical trajectory agrees to 1e-6 relative."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import load

pytestmark = pytest.mark.gpu
L_RTOL_FAST = 1e-6


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    yield capi.lib()
    capi.set_option("fast_foi", capi.FOI_AUTO)


def _model(**kw):
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(**kw)
    return capi.Model(mb.model_arrays(w)), [capi.Tables(mb.param_tables(w))]


def _hosp_model():
    """80 areas x 4 ages, weekly hospital populations: observations that read
    populations (the layout keeps two population buffers)."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.mbp_chain_model(80, 4)
    w.days = 60
    return capi.Model(mb.model_arrays(w)), [capi.Tables(mb.param_tables(w))]


CASES = {
    "100x3": lambda: _model(seed=20260201, narea=100, nage=3, days=60, name="mid"),
    "350x10": lambda: _model(seed=20260205, narea=350, nage=10, days=30, name="big350"),
    "hosp80x4": _hosp_model,
    "strains70x2x2": lambda: load("strain70_model")[1:3],
}


def _batched(dm, m, tabs, P, seed, **kw):
    capi.set_option("fast_foi", capi.FOI_BATCHED)
    try:
        db = capi.DeviceBatch(dm, capi.Batch(m, tabs, P, seed, form=capi.FORM_FAST, **kw))
    finally:
        capi.set_option("fast_foi", capi.FOI_AUTO)
    assert db.foi_path() == capi.FOI_BATCHED
    return db


@pytest.mark.parametrize("case", sorted(CASES))
def test_batched_follows_fp64_trajectories(built, case):
    m, tabs = CASES[case]()
    dm = capi.DeviceModel(m)
    P = 40
    g = dm.simulate(capi.Batch(m, tabs, P, 9, want_transnum=True, want_pop=True))
    db = _batched(dm, m, tabs, P, 9, want_transnum=True, want_pop=True)
    assert db.launches() == 3 * m.ndivision + 2          # per step: product, step kernel, observations
    f = db.run()
    db.close()
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.6, same.mean()
    assert all(np.array_equal(f.pop[p], g.pop[p]) for p in np.flatnonzero(same))
    np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
    dm.close()


def test_batched_parameter_set_per_particle(built):
    """ABC-SMC-like batch: every particle has its own parameter set (R0, 1/sigma,
    1/gamma from the priors), so the step kernel reloads a set's rates and table
    slices at nearly every work item; the particles follow the FP64 form's
    trajectories under their own sets."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260209, narea=100, nage=3, days=60, name="mid_groups")
    m = capi.Model(mb.model_arrays(w))
    P = 48
    R0, si, gi = synth.abc_smc_priors(np.random.default_rng(5), P)
    tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
    go = np.arange(P)
    dm = capi.DeviceModel(m)
    g = dm.simulate(capi.Batch(m, tabs, P, 31, group_of=go, want_transnum=True, want_pop=True))
    db = _batched(dm, m, tabs, P, 31, group_of=go, want_transnum=True, want_pop=True)
    f = db.run()
    db.close()
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.6, same.mean()
    np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
    dm.close()


def test_batched_uneven_tile_and_particle_counts(built):
    """Particle counts whose rows (particle x age) do not fill the last
    128-row tile, and more particles than the step kernel's CTAs (particles
    taken from the step counter in turn): every particle matches the same
    particle run in a batch of one."""
    m, tabs = CASES["100x3"]()
    dm = capi.DeviceModel(m)
    P = 1000                                    # 3000 rows: 23 full tiles and one of 56 rows
    db = _batched(dm, m, tabs, P, 21, want_pop=True)
    f = db.run()
    db.close()
    for p in (0, 1, 499, 998, 999):
        d1 = _batched(dm, m, tabs, 1, 21, stream_of=[p], want_pop=True)
        one = d1.run()
        d1.close()
        assert np.array_equal(one.pop[0], f.pop[p]), p
        np.testing.assert_allclose(one.L[0], f.L[p], rtol=L_RTOL_FAST)
    dm.close()


def test_batched_sections_carry_the_state(built):
    """Two sections [0, S/2) and [S/2, S) with the populations carried give the
    same trajectory and final populations as one run."""
    m, tabs = CASES["100x3"]()
    dm = capi.DeviceModel(m)
    P, S = 24, m.ndivision
    whole = _batched(dm, m, tabs, P, 5, want_transnum=True, want_pop=True).run()
    a = _batched(dm, m, tabs, P, 5, tf=S // 2, want_transnum=True, want_pop=True).run()
    b = _batched(dm, m, tabs, P, 5, ti=S // 2, pop_in=a.pop, want_transnum=True, want_pop=True).run()
    assert np.array_equal(np.concatenate([a.transnum, b.transnum], axis=1), whole.transnum)
    assert np.array_equal(b.pop, whole.pop)
    dm.close()


def test_batched_graph_replay_and_autotuner(built):
    """The batch's launches replayed as one CUDA graph give the same results as
    plain launches; the autotuner can choose the layout."""
    m, tabs = CASES["350x10"]()
    dm = capi.DeviceModel(m)
    P = 64
    db = _batched(dm, m, tabs, P, 3, want_pop=True)
    r1 = db.run()
    L1, pop1 = r1.L.copy(), r1.pop.copy()
    r2 = db.run_graph()
    assert np.array_equal(r2.pop, pop1)
    assert np.array_equal(r2.L, L1)
    db.close()
    chosen = dm.autotune(capi.Batch(m, tabs, 8 * 152, 3, form=capi.FORM_FAST))
    assert chosen in (capi.FOI_SIMT, capi.FOI_TENSOR, capi.FOI_BATCHED)
    dm.close()
