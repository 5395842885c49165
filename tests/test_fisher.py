"""Initial proposals from a Fisher matrix (wrappers/src/param.c:472-625), host
code of the library: the eigen rule against numpy's eigendecomposition, the
random-shift rule's box and reproducibility. No GPU needed."""
import numpy as np


def cov_and_fisher(D=4, seed=2):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(D, D))
    cov = A @ A.T + D * np.eye(D)
    return cov, np.linalg.inv(cov)


def test_eigen_rule(pmcg):
    D, K = 4, 6
    cov, F = cov_and_fisher(D)
    pos = np.array([0.1, -0.2, 0.3, 0.0])
    lo, hi = -np.full(D, 10.0), np.full(D, 10.0)
    prop = pmcg.MixMvdens(K, D)
    pmcg.fisher_proposal(prop, F, pos, lo, hi, kind=pmcg.FISHER_EIGEN, fshift=0.5, fvar=2.0)
    w, mu, L = prop.arrays()
    np.testing.assert_allclose(w, np.full(K, 1.0 / K))
    for k in range(K):
        np.testing.assert_allclose(L[k] @ L[k].T, 2.0 * cov, rtol=1e-10)
    lam, V = np.linalg.eigh(cov)
    order = np.argsort(-lam)
    for d in range(K // 2):
        r = 0.5 * lam[order[d]] / lam[order[0]] * V[:, order[d]]
        got = {tuple(np.round(mu[2 * d] - pos, 10)), tuple(np.round(mu[2 * d + 1] - pos, 10))}
        # -r then +r (the eigenvector's sign is arbitrary: compare the pair)
        assert got == {tuple(np.round(-r, 10)), tuple(np.round(r, 10))}
        np.testing.assert_allclose(mu[2 * d] + mu[2 * d + 1], 2 * pos, atol=1e-12)


def test_eigen_rule_refuses_more_than_two_per_direction(pmcg):
    D = 3
    _, F = cov_and_fisher(D)
    prop = pmcg.MixMvdens(2 * D + 1, D)
    try:
        pmcg.fisher_proposal(prop, F, np.zeros(D), -np.ones(D), np.ones(D), kind=pmcg.FISHER_EIGEN)
    except pmcg.PmcgError:
        return
    raise AssertionError("expected an error")


def test_random_shift_rule(pmcg):
    D, K = 4, 10
    cov, F = cov_and_fisher(D)
    pos = np.array([0.9, -0.9, 0.0, 0.5])
    lo, hi = -np.ones(D), np.ones(D)
    rng = pmcg.Rng(17)
    a = pmcg.fisher_proposal(pmcg.MixMvdens(K, D), F, pos, lo, hi, kind=pmcg.FISHER_RSHIFT, fshift=0.3, rng=rng)
    assert rng.calls == 1
    _, mu, L = a.arrays()
    assert np.all(mu >= lo) and np.all(mu <= hi)
    assert np.all(np.abs(mu - pos) <= 0.3 * (hi - lo) + 1e-15)
    assert len({tuple(m) for m in mu}) == K            # distinct shifts
    np.testing.assert_allclose(L[0] @ L[0].T, cov, rtol=1e-10)
    rng2 = pmcg.Rng(17)
    b = pmcg.fisher_proposal(pmcg.MixMvdens(K, D), F, pos, lo, hi, kind=pmcg.FISHER_RSHIFT, fshift=0.3, rng=rng2)
    np.testing.assert_array_equal(b.arrays()[1], mu)    # same seed and call: same proposal
