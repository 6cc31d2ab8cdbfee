"""The fast form's Poisson inversion searches the FP32 CDF two terms per pass
(sim_fast.cuh, poisson_fp32).  The pass computes the same products and sums in
the same order as a search of one term per pass, so it returns the same count;
both searches restated here in float32 arithmetic and compared on seeded
(mean, u) pairs across the inversion range, including the 63-term cap and
exhausted FP32 tails."""
import numpy as np

f32 = np.float32


def one_term(mean, u, rcp):
    p = f32(np.exp(f32(-mean)))
    F = p
    k = 0
    while u > F and k < 63:
        k += 1
        p = f32(f32(p * mean) * rcp[k])
        Fn = f32(F + p)
        if Fn == F:
            break
        F = Fn
    return k


def terms_per_pass(mean, u, rcp, n):
    p = f32(np.exp(f32(-mean)))
    F = p
    k = 0
    if not (u > F):
        return 0
    while k <= 63 - n:
        pt, Ft = [], []
        for j in range(n):
            pj = f32(f32((p if j == 0 else pt[j - 1]) * mean) * rcp[k + 1 + j])
            pt.append(pj)
            Ft.append(f32((F if j == 0 else Ft[j - 1]) + pj))
        for j in range(n):
            if Ft[j] == (F if j == 0 else Ft[j - 1]) or not (u > Ft[j]):
                return k + 1 + j
        k += n
        p, F = pt[-1], Ft[-1]
    while u > F and k < 63:
        k += 1
        p = f32(f32(p * mean) * rcp[k])
        Fn = f32(F + p)
        if Fn == F:
            break
        F = Fn
    return k


def test_two_terms_per_pass_give_the_same_counts():
    rcp = np.array([0.0] + [1.0 / k for k in range(1, 64)], dtype=np.float32)
    rng = np.random.default_rng(20261204)
    means = np.concatenate([rng.uniform(1e-4, 10.0, 4000), rng.uniform(9.0, 10.0, 1000)]).astype(np.float32)
    us = np.concatenate([rng.uniform(0, 1, 4000), 1.0 - rng.uniform(0, 1e-7, 1000)]).astype(np.float32)
    for n in (2, 3, 4):
        for m, u in zip(means, us):
            assert terms_per_pass(m, u, rcp, n) == one_term(m, u, rcp), (n, m, u)
