"""Parity at the two large workloads' full size (150 areas x 4 ages over 360
steps, and 350 areas x 10 ages over 1460 steps), not only on the small golden
fixtures:

* the plain FP64 form against the oracle, bit for bit: transition counts and
  populations identical, log-likelihood within 1e-12 relative
  (src/state.cc:596-638, src/obsmodel.cc:22-58);
* the fast form (FP32 SIMT force of infection, tensor-core force of infection
  per particle, and tensor cores batched over the particles in the
  step-synchronous layout, each forced) against the plain FP64 form as
  distributions, on
  independent variate streams: two-sample Kolmogorov-Smirnov and
  Anderson-Darling tests on the final epidemic size, the day of peak
  incidence and the log-likelihood, and every area's attack rate within
  Monte Carlo error;
* the trajectory-writing layout gives the same results as the layout that
  writes only L and the final populations (same particles, same streams)."""
import numpy as np
import pytest

from beep_gb300 import capi
from full_size import prior_tables, workload
from oracle_lib import oracle_simulate

pytestmark = pytest.mark.gpu
L_RTOL = 1e-12
E_TO_I = 1                          # transition index of E->I (daily cases)


@pytest.fixture(scope="module")
def built():
    from beep_gb300 import build
    build.build()
    yield capi.lib()
    capi.set_option("fast_foi", capi.FOI_AUTO)
    capi.set_option("fast_ctas_per_sm", 0)


@pytest.mark.parametrize("kind,P", [("abc_smc", 4), ("precision", 2)])
def test_plain_form_bit_exact_at_full_size(built, kind, P):
    w, m, t_true = workload(kind)
    tabs = prior_tables(w, P, 31) if kind == "abc_smc" else [t_true]
    go = np.arange(P) if kind == "abc_smc" else np.zeros(P, np.int32)
    seed = 20260777
    dm = capi.DeviceModel(m)
    g = dm.simulate(capi.Batch(m, tabs, P, seed, group_of=go, want_transnum=True, want_pop=True))
    dm.close()
    o = oracle_simulate(m, capi.Batch(m, tabs, P, seed, group_of=go, want_transnum=True, want_pop=True))
    assert g.transnum.sum() > 0
    for p in range(P):
        assert np.array_equal(g.transnum[p], o.transnum[p]), f"particle {p}: transition counts differ"
        assert np.array_equal(g.pop[p], o.pop[p]), f"particle {p}: populations differ"
    np.testing.assert_allclose(g.L, o.L, rtol=L_RTOL, atol=0)


def summaries(dm, m, tabs, P, seed, stream0, form, chunk):
    """Per particle: final epidemic size, day of peak incidence (E->I summed over
    areas and ages), log-likelihood, and each area's attack rate; with the
    trajectory-writing batch checked against the L-only batch."""
    S, A = m.ndivision, m.narea
    spd = int(round(1.0 / m.dt))
    pop0 = m.arr["pop_init"].reshape(A, m.ncomp, m.ndemocatpos)
    N = pop0.sum(axis=(1, 2)).astype(np.float64)
    S0 = pop0[:, 0, :].sum(axis=1).astype(np.float64)
    final, peak, L, attack = np.zeros(P), np.zeros(P), np.zeros(P), np.zeros((P, A))
    streams = stream0 + np.arange(P)
    # L and final populations in the layout the throughput measurement uses
    db = capi.DeviceBatch(dm, capi.Batch(m, tabs, P, seed, stream_of=streams, want_pop=True, form=form))
    b = db.run()
    path = db.foi_path()
    db.close()
    L[:] = b.L
    Send = b.pop[:, :, 0, :].sum(axis=2).astype(np.float64)
    attack[:] = (S0[None] - Send) / N[None]
    final[:] = (S0.sum() - Send.sum(axis=1))
    for k0 in range(0, P, chunk):
        n = min(chunk, P - k0)
        t = dm.simulate(capi.Batch(m, tabs, n, seed, stream_of=streams[k0:k0 + n], want_transnum=True, want_pop=True,
                                   form=form))
        # same trajectories; the fast form's observation terms may be spread over
        # another number of threads, so its L agrees to its own tolerance
        assert np.array_equal(t.pop, b.pop[k0:k0 + n]), "the trajectory layout changed the populations"
        np.testing.assert_allclose(t.L, b.L[k0:k0 + n], rtol=1e-6 if form == capi.FORM_FAST else 0, atol=0)
        inc = t.transnum[:, :, :, E_TO_I, :].sum(axis=(2, 3)).reshape(n, S // spd, spd).sum(axis=2)
        peak[k0:k0 + n] = inc.argmax(axis=1)
        del t
    return {"final": final, "peak": peak, "L": L, "attack": attack, "foi_path": path}


def assert_same_distribution(f, p, what):
    stats = pytest.importorskip("scipy.stats")
    ks = stats.ks_2samp(f, p).pvalue
    ad = stats.anderson_ksamp([f, p]).pvalue          # floored at 0.001 by scipy
    assert ks > 1e-3, f"{what}: KS p = {ks}"
    assert ad > 2e-3, f"{what}: Anderson-Darling p = {ad}"


def assert_attack_rates_agree(f, p):
    """Per-area mean attack rates within Monte Carlo error: every standardised
    difference below 4.5 (the family-wise bound for a few hundred areas) and at
    most 2% of areas beyond 3."""
    n1, n2 = len(f), len(p)
    d = f.mean(0) - p.mean(0)
    se = np.sqrt(f.var(0, ddof=1) / n1 + p.var(0, ddof=1) / n2)
    live = se > 0
    z = np.abs(d[live] / se[live])
    assert z.size > 0
    assert z.max() < 4.5, f"largest standardised attack-rate difference {z.max():.2f}"
    assert (z > 3).mean() <= 0.02, f"{(z > 3).mean():.3f} of areas beyond 3 standard errors"


@pytest.fixture(scope="module")
def plain_samples(built):
    """The plain FP64 form's summaries, 512 particles of each workload at the true parameters."""
    out = {}
    for kind, chunk in (("abc_smc", 128), ("precision", 64)):
        w, m, t_true = workload(kind)
        dm = capi.DeviceModel(m)
        out[kind] = summaries(dm, m, [t_true], 512, 20260901, 0, capi.FORM_PLAIN_FP64, chunk)
        dm.close()
    return out


@pytest.mark.parametrize("kind", ["abc_smc", "precision"])
@pytest.mark.parametrize("foi", [capi.FOI_SIMT, capi.FOI_TENSOR, capi.FOI_BATCHED])
def test_fast_form_distribution_at_full_size(plain_samples, kind, foi):
    w, m, t_true = workload(kind)
    capi.set_option("fast_foi", foi)
    try:
        dm = capi.DeviceModel(m)
        f = summaries(dm, m, [t_true], 512, 20260901, 10 ** 7, capi.FORM_FAST, 128 if kind == "abc_smc" else 64)
        dm.close()
    finally:
        capi.set_option("fast_foi", capi.FOI_AUTO)
    assert f["foi_path"] == foi
    p = plain_samples[kind]
    assert np.all(np.isfinite(f["L"]))
    for key in ("final", "peak", "L"):
        assert_same_distribution(f[key], p[key], f"{kind} {key}")
    assert_attack_rates_agree(f["attack"], p["attack"])
