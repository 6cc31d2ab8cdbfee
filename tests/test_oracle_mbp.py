"""The oracle's MBP restatement (Mbp::mbp, src/mbp.cc:252-330; State::likelihood,
src/state.cc:812-826) against the reference's own Mbp driven by the keyed
Poisson and binomial streams (fixtures made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

from beep_gb300 import capi
from golden_util import MBP_FIXTURES, MBP_VARIANTS, load, mbp_case, tn_checksums
from oracle_lib import oracle_lib, oracle_mbp

L_RTOL = 1e-12


@pytest.mark.parametrize("name", MBP_FIXTURES)
@pytest.mark.parametrize("v", range(MBP_VARIANTS))
def test_oracle_mbp_matches_reference(name, v):
    b, m, tabs, seed = load(name)
    gi, gp, si, sp, iu, simu = mbp_case(b, v)
    o = oracle_mbp(m, tabs, gi, gp, seed, si, sp, iu, simu, want_tn=True)
    p = f"mbp{v}."
    nc = len(gi)
    nt = b[p + "transnum_init"].shape[0]
    assert np.array_equal(o["tn_init"][:nt], b[p + "transnum_init"])
    assert np.array_equal(o["tn_prop"][:nt], b[p + "transnum_prop"])
    for k in range(nc):
        assert np.array_equal(tn_checksums(o["tn_init"][k]), b[p + "checksum"][k, 0])
        assert np.array_equal(tn_checksums(o["tn_prop"][k]), b[p + "checksum"][k, 1])
    for key in ("L_init", "L_prop", "Li_init", "Li_fixed"):
        np.testing.assert_allclose(o[key], b[p + key], rtol=L_RTOL, atol=0, err_msg=key)
    # EF = -2 L (State::set_EF, src/state.cc:95-98)
    np.testing.assert_allclose(-2 * o["L_prop"], b[p + "EF_prop"], rtol=L_RTOL)


def test_fixtures_exercise_every_coupled_draw():
    """Each kind of coupled draw occurs in the fixtures: n + Poisson(m'-m),
    n kept (m' = m) and Binomial(n, m'/m) thinning."""
    b, m, tabs, seed = load("tiny_mbp")
    gi, gp, si, sp, iu, simu = mbp_case(b, 0)
    o = oracle_mbp(m, tabs, gi, gp, seed, si, sp, iu, simu, want_tn=True)
    d = o["tn_prop"].astype(np.int64) - o["tn_init"]
    assert (d > 0).any() and (d < 0).any() and (d == 0).any()


def test_binomial_sampler_distribution():
    """The keyed binomial thinning draw (inversion below n q = 10, BTRS above)
    follows Binomial(n, p): chi-square against the exact pmf."""
    stats = pytest.importorskip("scipy.stats")
    L = oracle_lib()
    for n, p in ((8, 0.3), (40, 0.5), (1000, 0.93), (100000, 0.3)):
        N = 40000
        x = np.array([L.beep_oracle_binomial(p, n, 99, j % 997, j % 6, j // 5982, 7) for j in range(N)])
        assert x.min() >= 0 and x.max() <= n
        pmf = stats.binom.pmf(np.arange(n + 1), n, p)
        cnt = np.bincount(x, minlength=n + 1)
        keep = pmf * N >= 20
        e = np.append(pmf[keep] * N, pmf[~keep].sum() * N)
        o = np.append(cnt[keep], cnt[~keep].sum())
        if e[-1] < 1:
            e, o = e[:-1], o[:-1]
        chi = ((o - e) ** 2 / e).sum()
        assert stats.chi2.sf(chi, len(e) - 1) > 1e-3, (n, p)
    # the edge cases of the thinning: nothing to thin, p = 1, p = 0
    assert L.beep_oracle_binomial(0.4, 0, 1, 0, 0, 0, 0) == 0
    assert L.beep_oracle_binomial(1.0, 17, 1, 0, 0, 0, 0) == 17
    assert L.beep_oracle_binomial(0.0, 17, 1, 0, 0, 0, 0) == 0


def test_acceptance_matches_reference():
    """Mbp::get_al (src/mbp.cc:334-361) in INVT mode with invT = 1."""
    b, m, tabs, seed = load("tiny_mbp")
    for v in range(MBP_VARIANTS):
        p = f"mbp{v}."
        for k in range(int(b["mbp.nchain"][0])):
            ef_p, ef_i, pr_p, pr_i = b[p + "EF_prop"][k], b[p + "EF_init"][k], b[p + "Pr_prop"][k], b[p + "Pr_init"][k]
            al = min(1.0, np.exp(-0.5 * (ef_p - ef_i) + pr_p - pr_i))
            np.testing.assert_allclose(al, b[p + "al"][k], rtol=1e-12)
