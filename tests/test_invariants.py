"""Size-independent properties of a trajectory, the checks BEEP's own
State::check makes (src/state_check.cc:8-99), applied at the workloads' full
per-particle sizes: every count is non-negative, no transition leaves an empty
compartment, the populations follow update_pop from the counts, and each
area's population of every demographic position is conserved.  The checker
is pinned on the oracle (CPU); the fast form is checked on the GPU, where its
trajectories at these sizes mostly differ from the FP64 ones."""
import numpy as np
import pytest

from beep_gb300 import capi, model_builder as mb, synth


def check_trajectory(m, transnum, pop_traj, pop_final):
    """transnum [S][A][T][DP], pop_traj [S][A][C][DP] (start of each step), pop_final [A][C][DP]."""
    assert m.nstrain == 1                              # no strain shift between steps
    frm = np.asarray(m.arr["trans_from"])
    to = np.asarray(m.arr["trans_to"])
    tn = transnum.astype(np.int64)
    pp = np.concatenate([pop_traj, pop_final[None]], 0).astype(np.int64)
    assert (tn >= 0).all(), "negative transition count"
    src = pp[:-1][:, :, frm, :]                      # [S][A][T][DP] population of each source
    assert (tn[src <= 0] == 0).all(), "transition from an empty compartment"
    flow = np.zeros_like(pp[:-1])
    np.add.at(flow, (slice(None), slice(None), frm, slice(None)), -tn)
    np.add.at(flow, (slice(None), slice(None), to, slice(None)), tn)
    assert np.array_equal(pp[1:], pp[:-1] + flow), "populations do not follow update_pop"
    tot = pp.sum(2)                                   # [S+1][A][DP]
    assert (tot == tot[0]).all(), "population not conserved"


def _abc_model(nage=4, narea=150):
    w = synth.abc_smc_large(narea=narea, nage=nage)
    return capi.Model(mb.model_arrays(w)), w


def test_checker_on_oracle_trajectories():
    from oracle_lib import oracle_simulate
    m, w = _abc_model()
    R0, si, gi = synth.abc_smc_priors(np.random.default_rng(1), 2)
    tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
    b = oracle_simulate(m, capi.Batch(m, tabs, 2, 11, group_of=np.arange(2), want_transnum=True, want_pop_traj=True,
                                      want_pop=True))
    for p in range(2):
        check_trajectory(m, b.transnum[p], b.pop_traj[p], b.pop[p])
    # and it notices a count moved by one
    bad = b.transnum[0].copy()
    s, c, tr, dp = np.argwhere(bad > 0)[0]
    bad[s, c, tr, dp] -= 1
    with pytest.raises(AssertionError):
        check_trajectory(m, bad, b.pop_traj[0], b.pop[0])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["abc_smc", "precision"])
def test_fast_form_trajectories_at_full_size(kind):
    """The ABC-SMC generation's model (150 x 4, 360 steps, several particles per
    SM) and the precision model (350 x 10, 1460 steps, tensor-core FOI)."""
    if kind == "abc_smc":
        m, w = _abc_model()
        R0, si, gi = synth.abc_smc_priors(np.random.default_rng(2), 8)
        tabs = [capi.Tables(t) for t in mb.param_tables_batch(w, R0, si, gi)]
        P, go = 8, np.arange(8)
    else:
        w = synth.precision_large()
        m = capi.Model(mb.model_arrays(w))
        tabs = [capi.Tables(mb.param_tables(w))]
        P, go = 2, np.zeros(2, np.int32)
    dm = capi.DeviceModel(m)
    b = dm.simulate(capi.Batch(m, tabs, P, 21, group_of=go, want_transnum=True, want_pop_traj=True, want_pop=True,
                               form=capi.FORM_FAST))
    dm.close()
    for p in range(P):
        check_trajectory(m, b.transnum[p], b.pop_traj[p], b.pop[p])
