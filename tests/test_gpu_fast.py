"""Fast (mixed-precision) form: same keyed streams as the FP64 form, so most
particles follow the FP64 trajectory exactly; the log-likelihood of a
trajectory agrees with the FP64 evaluation of that same trajectory to 1e-6
relative; and the distribution of outcomes matches the oracle."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import FAST_FIXTURES, load
from oracle_lib import oracle_simulate

pytestmark = pytest.mark.gpu
L_RTOL_FAST = 1e-6


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    return capi.lib()


def fp64_loglik_of(m, tabs, transnum, pop_traj, seed):
    """FP64 log-likelihood of given trajectories: replay them through the oracle's
    observation model by simulating with the plain form and comparing -- here we
    recompute it directly from the counts in numpy, in the reference's order."""
    from oracle_lib import oracle_lib  # noqa: F401
    arr = m.arr
    ptr, cells = arr["obs_cell_ptr"], arr["obs_cells"]
    si, sf = arr["obs_sett_i"], arr["obs_sett_f"]
    S = transnum.shape[0]
    tn = transnum.reshape(S, -1).astype(np.float64)
    pp = pop_traj.reshape(S, -1).astype(np.float64)
    L = 0.0
    for o in range(m.nobs):
        v = 0.0
        for s in range(si[o], sf[o]):
            for q in range(ptr[o], ptr[o + 1]):
                c = int(cells[q])
                v += tn[s, c] if c >= 0 else pp[s, -1 - c]
        y, sd = arr["obs_value"][o], arr["obs_sd"][o]
        var = sd * sd
        L += -0.5 * np.log(2 * np.pi * var) - (y - v) ** 2 / (2 * var)
    return L


@pytest.mark.parametrize("name", FAST_FIXTURES)
def test_fast_follows_fp64_trajectories(built, name):
    b, m, tabs, seed = load(name)
    P = 64
    dm = capi.DeviceModel(m)
    f = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True, want_pop=True, form=capi.FORM_FAST))
    g = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True, want_pop=True))
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.75, same.mean()
    # identical trajectories: log-likelihood within the FP32-compensated tolerance
    np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
    dm.close()


@pytest.fixture
def draws_option(built):
    yield capi.set_option
    capi.set_option("fast_parallel_draws", 0)


@pytest.mark.parametrize("name", ["tiny_sim", "c0_sim", "strain_sim", "obsmodel_sim", "features_sim", "pred_sim", "oneage_sim"])
def test_parallel_draws_give_the_same_trajectories(draws_option, name):
    """Small models: a step's draws one per (transition, column) thread draw the
    same keyed variates from the same means as the column threads drawing their
    transitions one after another, so counts, populations and log-likelihoods are
    identical (population updates are integer atomics, whose order does not
    matter)."""
    b, m, tabs, seed = load(name)
    dm = capi.DeviceModel(m)
    res = []
    for opt in (1, 2):
        draws_option("fast_parallel_draws", opt)
        r = dm.simulate(capi.Batch(m, tabs, 24, seed, want_transnum=True, want_pop=True, form=capi.FORM_FAST))
        res.append((r.transnum.copy(), r.pop.copy(), r.L.copy()))
    for a, c in zip(*res):
        assert np.array_equal(a, c)
    dm.close()


def test_fast_loglik_matches_fp64_of_same_trajectory(built):
    b, m, tabs, seed = load("tiny_sim")
    P = 16
    dm = capi.DeviceModel(m)
    f = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True, want_pop_traj=True, form=capi.FORM_FAST))
    for p in range(P):
        L64 = fp64_loglik_of(m, tabs, f.transnum[p], f.pop_traj[p], seed)
        assert abs(f.L[p] - L64) <= L_RTOL_FAST * abs(L64)
    dm.close()


def test_fast_distribution_matches_oracle(built):
    stats = pytest.importorskip("scipy.stats")
    b, m, tabs, seed = load("c0_sim")
    P = 400
    dm = capi.DeviceModel(m)
    f = dm.simulate(capi.Batch(m, tabs, P, seed + 99, stream_of=np.arange(P) + 10 ** 6, want_pop=True,
                               form=capi.FORM_FAST))
    o = oracle_simulate(m, capi.Batch(m, tabs, P, seed + 7, want_pop=True))
    # final epidemic size (recovered + dead) and log-likelihood: same distribution
    fs_f = f.pop[:, :, 4:6, :].sum(axis=(1, 2, 3))
    fs_o = o.pop[:, :, 4:6, :].sum(axis=(1, 2, 3))
    assert stats.ks_2samp(fs_f, fs_o).pvalue > 1e-3
    assert stats.ks_2samp(f.L, o.L).pvalue > 1e-3
    dm.close()


def test_fast_large_model_keeps_state_in_global_memory(built):
    """A model whose per-particle state exceeds shared memory (200 areas x 8
    ages) runs the fast form with its state in global memory: same streams,
    trajectories follow the FP64 form."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260200, narea=200, nage=8, days=30, name="big")
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    dm = capi.DeviceModel(m)
    P = 24
    f = dm.simulate(capi.Batch(m, [t], P, 5, want_transnum=True, want_pop=True, form=capi.FORM_FAST))
    g = dm.simulate(capi.Batch(m, [t], P, 5, want_transnum=True, want_pop=True))
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.5, same.mean()
    np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
    dm.close()


@pytest.fixture
def foi_option(built):
    yield capi.set_option
    capi.set_option("fast_foi", capi.FOI_AUTO)


def test_tensor_core_foi_follows_fp64(foi_option):
    """The force of infection on the tensor cores (split BF16, FP32 accumulation)
    and the FP32 SIMT contraction both keep the fast form on the FP64
    trajectories of a 100-area x 3-age model."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260201, narea=100, nage=3, days=60, name="mid")
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    dm = capi.DeviceModel(m)
    P = 48
    g = dm.simulate(capi.Batch(m, [t], P, 9, want_transnum=True, want_pop=True))
    res = {}
    for mode in (capi.FOI_SIMT, capi.FOI_TENSOR):
        foi_option("fast_foi", mode)
        db = capi.DeviceBatch(dm, capi.Batch(m, [t], P, 9, want_transnum=True, want_pop=True, form=capi.FORM_FAST))
        assert db.foi_path() == mode
        f = db.run()
        db.close()
        same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
        assert same.mean() >= 0.6, (mode, same.mean())
        np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
        res[mode] = f
    both = np.array([np.array_equal(res[1].transnum[p], res[2].transnum[p]) for p in range(P)])
    assert both.mean() >= 0.6, both.mean()
    dm.close()


def test_tensor_core_foi_distribution_matches_oracle(foi_option):
    stats = pytest.importorskip("scipy.stats")
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260202, narea=90, nage=4, days=50, name="mid2")
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    foi_option("fast_foi", capi.FOI_TENSOR)
    dm = capi.DeviceModel(m)
    P = 300
    db = capi.DeviceBatch(dm, capi.Batch(m, [t], P, 77, stream_of=np.arange(P) + 5 * 10 ** 5, want_pop=True,
                                         form=capi.FORM_FAST))
    assert db.foi_path() == capi.FOI_TENSOR
    f = db.run()
    db.close()
    o = oracle_simulate(m, capi.Batch(m, [t], P, 78, want_pop=True))
    fs_f = f.pop[:, :, 4:6, :].sum(axis=(1, 2, 3))
    fs_o = o.pop[:, :, 4:6, :].sum(axis=(1, 2, 3))
    assert stats.ks_2samp(fs_f, fs_o).pvalue > 1e-3
    assert stats.ks_2samp(f.L, o.L).pvalue > 1e-3
    dm.close()


@pytest.fixture
def ctas_option(built):
    yield capi.set_option
    capi.set_option("fast_ctas_per_sm", 0)


def test_several_particles_per_sm_follow_fp64(ctas_option):
    """Two to four 320-thread CTAs per SM (smaller register budget, more warps)
    run the same arithmetic per column as one 640-thread CTA: the particles
    follow the FP64 trajectories and score them within the fast-form tolerance,
    whichever layout runs; the automatic choice takes four for a batch that
    fills the SMs four deep and one for a small batch."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260203, narea=100, nage=4, days=60, name="mid3")
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    dm = capi.DeviceModel(m)
    P = 96
    g = dm.simulate(capi.Batch(m, [t], P, 11, want_transnum=True, want_pop=True))
    res = {}
    for k in (0, 1, 2, 3, 4):
        ctas_option("fast_ctas_per_sm", k)
        db = capi.DeviceBatch(dm, capi.Batch(m, [t], P, 11, want_transnum=True, want_pop=True, form=capi.FORM_FAST))
        assert db.ctas_per_sm() == (1 if k == 0 else k), (k, db.ctas_per_sm())   # automatic: 96 particles fill no SM 4-deep
        assert db.foi_path() == capi.FOI_SIMT
        f = db.run()
        db.close()
        same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
        assert same.mean() >= 0.6, (k, same.mean())
        np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
        res[k] = f
    # the multi-CTA layouts read the area matrix the same way: identical results
    for k in (3, 4):
        assert np.array_equal(res[k].transnum, res[2].transnum)
        assert np.array_equal(res[k].L, res[2].L)
    # automatic choice by expected waves: four per SM once the batch fills them
    ctas_option("fast_ctas_per_sm", 0)
    for P2, want in ((152, 1), (4 * 152 * 2, 4)):
        db = capi.DeviceBatch(dm, capi.Batch(m, [t], P2, 11, form=capi.FORM_FAST))
        assert db.ctas_per_sm() == want, (P2, db.ctas_per_sm())
        db.close()
    dm.close()


def test_several_particles_per_sm_with_state_in_global_memory(ctas_option):
    """A model whose per-particle state lives in global memory (300 areas x 10
    ages) runs two or three 320-thread particles per SM with only the
    infectious counts, force of infection and slots on chip, and follows the
    FP64 form."""
    from beep_gb300 import model_builder as mb, synth
    w = synth.seir_hd_small(seed=20260204, narea=300, nage=10, days=20, name="big2")
    m = capi.Model(mb.model_arrays(w))
    t = capi.Tables(mb.param_tables(w))
    dm = capi.DeviceModel(m)
    P = 24
    g = dm.simulate(capi.Batch(m, [t], P, 5, want_transnum=True, want_pop=True))
    ctas_option("fast_foi", capi.FOI_SIMT)
    try:
        for k in (1, 4):
            ctas_option("fast_ctas_per_sm", k)
            db = capi.DeviceBatch(dm, capi.Batch(m, [t], P, 5, want_transnum=True, want_pop=True, form=capi.FORM_FAST))
            assert db.ctas_per_sm() == 1 if k == 1 else db.ctas_per_sm() in (2, 3)
            f = db.run()
            db.close()
            same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
            assert same.mean() >= 0.5, (k, same.mean())
            np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
    finally:
        ctas_option("fast_foi", capi.FOI_AUTO)
    dm.close()


def test_several_particles_per_sm_with_two_strains(ctas_option):
    """Two strains (70 areas x 2 ages x 2 strains, 280 columns; model and tables
    from the reference) in the four-per-SM layout: the same draws as one
    640-thread CTA per SM, and the particles follow the FP64 form."""
    b, m, tabs, seed = load("strain70_model")
    assert m.nstrain == 2 and m.narea * m.ndemocatpos > 256
    dm = capi.DeviceModel(m)
    P = 48
    g = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True))
    res = {}
    for k in (1, 4):
        ctas_option("fast_ctas_per_sm", k)
        db = capi.DeviceBatch(dm, capi.Batch(m, tabs, P, seed, want_transnum=True, form=capi.FORM_FAST))
        assert db.ctas_per_sm() == k
        res[k] = db.run()
        db.close()
    assert np.array_equal(res[1].transnum, res[4].transnum)
    np.testing.assert_allclose(res[4].L, res[1].L, rtol=1e-6)
    same = np.array([np.array_equal(res[4].transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.5, same.mean()
    np.testing.assert_allclose(res[4].L[same], g.L[same], rtol=L_RTOL_FAST)
    dm.close()


def test_tensor_core_foi_with_two_strains(foi_option):
    """The tensor-core FOI with two strains (each strain's counts in its own
    32 rows of the M = 64 operand) keeps the fast form on the FP64
    trajectories of the 70-area two-strain reference model."""
    b, m, tabs, seed = load("strain70_model")
    dm = capi.DeviceModel(m)
    P = 48
    g = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True))
    foi_option("fast_foi", capi.FOI_TENSOR)
    db = capi.DeviceBatch(dm, capi.Batch(m, tabs, P, seed, want_transnum=True, form=capi.FORM_FAST))
    assert db.foi_path() == capi.FOI_TENSOR
    f = db.run()
    db.close()
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.5, same.mean()
    np.testing.assert_allclose(f.L[same], g.L[same], rtol=L_RTOL_FAST)
    dm.close()
