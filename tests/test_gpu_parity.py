"""CUDA plain FP64 form vs the reference (golden fixtures) and the oracle,
called through the C ABI (libbeep_gpu.so).  Bar: transition counts and
populations bit-exact; log-likelihood within 1e-12 relative."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import FIXTURES, PF_FIXTURES, checksums, load
from oracle_lib import oracle_simulate

pytestmark = pytest.mark.gpu
L_RTOL = 1e-12


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    return capi.lib()


@pytest.mark.parametrize("name", FIXTURES)
def test_full_simulation_matches_reference(built, name):
    b, m, tabs, seed = load(name)
    P = int(b["npart"][0])
    nt = b["g0.transnum"].shape[0]
    dm = capi.DeviceModel(m)
    bt = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True, want_pop_traj=True, want_pop=True))
    assert np.array_equal(bt.transnum[:nt], b["g0.transnum"])
    assert np.array_equal(bt.pop_traj[:nt], b["g0.pop"])
    for p in range(P):
        assert np.array_equal(checksums(bt.transnum[p], bt.pop_traj[p]), b["g0.checksum"][p])
    np.testing.assert_allclose(bt.L, b["g0.L"], rtol=L_RTOL, atol=0)
    dm.close()


@pytest.mark.parametrize("name", PF_FIXTURES)
def test_sections_match_reference(built, name):
    b, m, tabs, seed = load(name)
    P = int(b["npart"][0])
    dm = capi.DeviceModel(m)
    pop = None
    tns = []
    for k, (ti, tf) in enumerate(m.sections):
        bt = dm.simulate(capi.Batch(m, tabs, P, seed, ti=ti, tf=tf, pop_in=pop, want_pop=True, want_transnum=True))
        np.testing.assert_allclose(bt.L, b["g0.L_section"][:, k], rtol=L_RTOL, atol=1e-12)
        pop = bt.pop
        tns.append(bt.transnum)
    tn = np.concatenate(tns, axis=1)
    assert np.array_equal(tn[:b["g0.transnum"].shape[0]], b["g0.transnum"])
    dm.close()


def test_many_particles_and_groups_match_oracle(built):
    """Mixed parameter sets (group_of) and caller-chosen streams over 200
    particles: identical counts and populations to the oracle."""
    b, m, tabs, seed = load("c0_sim")
    t2 = capi.Tables({k: (v * 1.3 if k == "g0.beta_rows" else v) for k, v in b.items()}, "g0.")
    P = 200
    rng = np.random.default_rng(5)
    group_of = rng.integers(0, 2, P)
    stream_of = rng.permutation(100000)[:P].astype(np.uint32)
    dm = capi.DeviceModel(m)
    g = dm.simulate(capi.Batch(m, [tabs[0], t2], P, seed, group_of=group_of, stream_of=stream_of,
                               want_pop=True, want_transnum=True))
    o = oracle_simulate(m, capi.Batch(m, [tabs[0], t2], P, seed, group_of=group_of, stream_of=stream_of,
                                      want_pop=True, want_transnum=True))
    assert np.array_equal(g.transnum, o.transnum)
    assert np.array_equal(g.pop, o.pop)
    np.testing.assert_allclose(g.L, o.L, rtol=L_RTOL, atol=0)
    dm.close()


def test_device_errors_are_statuses(built):
    b, m, tabs, seed = load("tiny_sim")
    dm = capi.DeviceModel(m)
    with pytest.raises(capi.BeepError) as e:
        dm.simulate(capi.Batch(m, tabs, 4, seed, ti=5, tf=3))
    assert e.value.status == 1
    bad = capi.Tables({k: (v * np.nan if k == "g0.beta_rows" else v) for k, v in b.items()}, "g0.")
    with pytest.raises(capi.BeepError) as e:
        dm.simulate(capi.Batch(m, [bad], 2, seed))
    assert e.value.status == 2
    # the model stays usable after an error
    ok = dm.simulate(capi.Batch(m, tabs, 2, seed))
    np.testing.assert_allclose(ok.L, b["g0.L"][:2], rtol=L_RTOL)
    dm.close()


@pytest.mark.parametrize("name", PF_FIXTURES)
def test_particle_filter_matches_reference(built, name):
    """Device particle filter (plain form) vs the reference's own bootstrap and
    ancestor swap: identical ancestors, estimate and section terms to 1e-12."""
    b, m, tabs, seed = load(name)
    N = b["g0.pf.ancestors"].shape[1]
    dm = capi.DeviceModel(m)
    ll, lls, L, anc, lin = dm.pf_loglik(tabs[0], N, seed, int(b["g0.pf.stream"][0]), float(b["g0.pf.invT"][0]),
                                        m.sections, lineage=True)
    assert np.array_equal(anc, b["g0.pf.ancestors"])
    assert np.array_equal(lin, b["g0.pf.lineage_transnum"])     # Mpi::particle_sample
    np.testing.assert_allclose(L, b["g0.pf.L_section"], rtol=L_RTOL, atol=1e-12)
    np.testing.assert_allclose(lls, b["g0.pf.obprob_section"], rtol=L_RTOL, atol=1e-12)
    np.testing.assert_allclose(ll, b["g0.pf.obprob"][0], rtol=L_RTOL)
    dm.close()


def test_particle_filter_fast_form_and_oracle(built):
    """The filter with the fast form runs to a finite estimate, and the plain
    form agrees with the oracle's filter on a larger particle count."""
    from oracle_lib import oracle_pf
    b, m, tabs, seed = load("c0_pf")
    dm = capi.DeviceModel(m)
    N = 256
    llg, _, _, ancg, ling = dm.pf_loglik(tabs[0], N, seed + 3, 77, 1.0, m.sections, lineage=True)
    llo, _, _, anco, lino = oracle_pf(m, tabs[0], N, seed + 3, 77, 1.0, m.sections, lineage=True)
    assert np.array_equal(ancg, anco)
    assert np.array_equal(ling, lino)
    np.testing.assert_allclose(llg, llo, rtol=L_RTOL)
    llf, _, _, ancf, linf = dm.pf_loglik(tabs[0], N, seed + 3, 77, 1.0, m.sections, form=capi.FORM_FAST, lineage=True)
    assert np.isfinite(llf) and ancf.min() >= 0 and ancf.max() < N
    # the fast form's lineage is a full trajectory: counts in every section, infections included
    assert linf.min() >= 0
    for ti, tf in m.sections:
        assert linf[ti:tf].sum() > 0
    dm.close()


def test_particle_filter_repeated_calls_reuse_prepared_sections(built):
    """Calls of the same shape reuse the prepared section batches, with only the
    tables and keys changed: each result equals that of a fresh model, in both
    forms, with other parameter sets, seeds and shapes between the calls."""
    b, m, tabs, seed = load("c0_pf")
    N = 64
    secs = m.sections
    # a second parameter set: the transition rates and R(t) rows scaled
    arr = dict(tabs[0].arr)
    arr = {k: v.reshape(tabs[0].shapes[k]) for k, v in arr.items() if k in tabs[0].shapes}
    arr["transrate"] = arr["transrate"] * 1.1
    arr["beta_rows"] = arr["beta_rows"] * 0.9
    t2 = capi.Tables(arr)
    calls = [(tabs[0], seed + 1, capi.FORM_PLAIN_FP64, N), (t2, seed + 2, capi.FORM_PLAIN_FP64, N),
             (tabs[0], seed + 3, capi.FORM_FAST, N), (t2, seed + 4, capi.FORM_FAST, N),
             (tabs[0], seed + 5, capi.FORM_FAST, 32), (t2, seed + 6, capi.FORM_FAST, N)]
    dm = capi.DeviceModel(m)
    reused = [dm.pf_loglik(t, n, sd, 9, 1.0, secs, form=f) for t, sd, f, n in calls]
    dm.close()
    for (t, sd, f, n), got in zip(calls, reused):
        fresh = capi.DeviceModel(m)
        want = fresh.pf_loglik(t, n, sd, 9, 1.0, secs, form=f)
        fresh.close()
        assert got[0] == want[0]
        assert np.array_equal(got[1], want[1]) and np.array_equal(got[2], want[2]) and np.array_equal(got[3], want[3])


def test_prediction_multipliers_match_oracle(built):
    """PREDICTION-mode modifications (efoi_mult, transmean_mult; src/state.cc:415,
    446-453): the plain form equals the oracle restatement bit for bit, the fast
    form follows it, and all-ones multipliers change nothing."""
    from oracle_lib import oracle_simulate
    b, m, tabs, seed = load("c0_sim")
    rng = np.random.default_rng(11)
    S, A, T, DP, NS = m.ndivision, m.narea, m.ntrans, m.ndemocatpos, m.nstrain
    base = {k: v for k, v in b.items() if k.startswith("g0.")}
    arr = {k[3:]: v for k, v in base.items()}
    arr["efoi_mult"] = rng.uniform(0.5, 1.5, (S, A, NS))
    tm = np.ones((S, A, T, DP))
    tm[S // 3:] *= rng.uniform(0.6, 1.1, (S - S // 3, A, T, DP))   # an intervention from a third of the horizon
    arr["transmean_mult"] = tm
    tmod = capi.Tables(arr)
    P = 24
    dm = capi.DeviceModel(m)
    g = dm.simulate(capi.Batch(m, [tmod], P, seed, want_transnum=True))
    o = oracle_simulate(m, capi.Batch(m, [tmod], P, seed, want_transnum=True))
    assert np.array_equal(g.transnum, o.transnum)
    np.testing.assert_allclose(g.L, o.L, rtol=1e-12)
    plain0 = dm.simulate(capi.Batch(m, tabs, P, seed, want_transnum=True))
    assert not np.array_equal(g.transnum, plain0.transnum)          # the modification acts
    ones = dict(arr)
    ones["efoi_mult"] = np.ones((S, A, NS))
    ones["transmean_mult"] = np.ones((S, A, T, DP))
    u = dm.simulate(capi.Batch(m, [capi.Tables(ones)], P, seed, want_transnum=True))
    assert np.array_equal(u.transnum, plain0.transnum)
    f = dm.simulate(capi.Batch(m, [tmod], P, seed, want_transnum=True, form=capi.FORM_FAST))
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.6, same.mean()
    dm.close()


def test_negative_binomial_observations_match_oracle(built):
    """Negative-binomial observations (ObservationModel::obs_prob with
    negative_binomial_probability, src/obsmodel.cc:245-305,
    src/utils.cc:124-127), plain values and censored ones: the reference's
    TOML parser rejects every 'negbin' string (src/inputs.cc:455-460), so the
    observation-model fixture's Poisson entries are switched to negative
    binomial here; the plain form equals the oracle restatement, the fast form
    follows it."""
    from oracle_lib import oracle_simulate
    b, m, tabs, seed = load("obsmodel_sim")
    arr = dict(b)                                                     # the bundle's model arrays
    pois = np.asarray(arr["obs_model"]) == 2
    assert pois.any()
    assert (np.asarray(arr["obs_value_kind"])[pois] == 2).any()
    arr["obs_model"] = np.where(pois, 3, arr["obs_model"]).astype(np.int32)
    arr["obs_shape"] = np.where(pois, 4.5, arr["obs_shape"])
    mn = capi.Model(arr)
    P = 16
    dm = capi.DeviceModel(mn)
    g = dm.simulate(capi.Batch(mn, tabs, P, seed, want_transnum=True))
    o = oracle_simulate(mn, capi.Batch(mn, tabs, P, seed, want_transnum=True))
    assert np.array_equal(g.transnum, o.transnum)
    np.testing.assert_allclose(g.L, o.L, rtol=1e-12)
    gp = capi.DeviceModel(m).simulate(capi.Batch(m, tabs, P, seed))
    assert np.abs(gp.L - g.L).min() > 0.1                              # the model changed every likelihood
    f = dm.simulate(capi.Batch(mn, tabs, P, seed, want_transnum=True, form=capi.FORM_FAST))
    same = np.array([np.array_equal(f.transnum[p], g.transnum[p]) for p in range(P)])
    assert same.mean() >= 0.6, same.mean()
    np.testing.assert_allclose(f.L[same], g.L[same], rtol=1e-6)
    dm.close()


def test_prediction_from_loaded_samples_matches_reference(built):
    """The reference's prediction mode on samples written by beep_gb300.samples
    (State::load, then State::simulate from the modifications' start under the
    modification multipliers, src/simulate.cc:142-165, src/state.cc:415,446-453):
    the plain form, started from the loaded populations, gives the reference's
    counts and final populations bit for bit; the fast form follows them."""
    from golden_util import prediction_runs
    b, m, tabs, seed = load("pred_sim")
    dm = capi.DeviceModel(m)
    runs = prediction_runs(b)
    for r in runs:
        g = dm.simulate(capi.Batch(m, [r["tables"]], 1, seed, ti=r["ti"], pop_in=r["pop_ti"][None],
                                   stream_of=[r["stream"]], want_transnum=True, want_pop=True))
        assert np.array_equal(g.transnum[0], r["transnum"])
        assert np.array_equal(g.pop[0], r["pop_end"])
    same = 0
    for r in runs:
        f = dm.simulate(capi.Batch(m, [r["tables"]], 1, seed, ti=r["ti"], pop_in=r["pop_ti"][None],
                                   stream_of=[r["stream"]], want_transnum=True, form=capi.FORM_FAST))
        same += int(np.array_equal(f.transnum[0], r["transnum"]))
    assert same >= len(runs) // 2, same
    dm.close()
