"""Importance sampling of an existing sample with another posterior
(exec/importance_sample.c) and device weighted moments, through the C ABI,
against the FP64 oracle and numpy."""
import numpy as np
import pytest

from cosmopmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_importance_sample_sn_matches_oracle(pmcg, oracle):
    """Weights := log posterior (flat box prior + SN likelihood); flg = 0 outside the
    box and on a loitering cosmology."""
    wl = W.sn_workload(nsn=120)
    sn = wl["sn"]
    post = pmcg.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(sn)
    rng = np.random.default_rng(8)
    N = 3001
    X = rng.uniform(wl["bmin"], wl["bmax"], (N, 6))
    X[0] = [0.0, 1.5, -3.0, -19.1, 0.1, 3.0]   # loitering
    X[1, 0] = wl["bmax"][0] + 0.5              # outside the box
    ps = pmcg.PmcSimu(N, 6)
    ps.X[:] = X
    ps.host_modified()
    count = ps.importance_sample(post)
    ref, ok = oracle.sn_loglike(sn, X)
    inside = np.all((X >= wl["bmin"]) & (X <= wl["bmax"]), axis=1)
    good = (ok == 1) & inside
    np.testing.assert_array_equal(ps.flg == 1, good)
    assert count == good.sum() and ps.s.isLog == 1
    logpr = -np.sum(np.log(wl["bmax"] - wl["bmin"]))
    np.testing.assert_allclose(ps.weights[good], ref[good] + logpr, rtol=1e-11, atol=1e-8)
    assert ps.s.maxW == pytest.approx(np.max(ref[good] + logpr), rel=1e-12)


def test_importance_reweighting_from_a_sample_file(pmcg, oracle, tmp_path):
    """A PMC sample written to file, read back, re-weighted by a second likelihood
    (the importance_sample flow): combined weights = old * new, as the reference
    combines them (exec/importance_sample.c:265-284)."""
    D, K = 4, 3
    wl = W.mixture_workload(D=D, K=K, Kt=1, nu=-1, seed=21, prop_hi=1.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()
    target = pmcg.MixMvdens.from_arrays(wt, mut, cov=covt, df=-1).cholesky()
    post = pmcg.Posterior(D).add_mix(target)
    N = 20000
    ps = pmcg.PmcSimu(N, D)
    rng = pmcg.Rng(5)
    pmcg.simulate_mix_mvdens(ps, prop, rng, None)
    pmcg.importance_weights(ps, prop, post, 1.0)
    pmcg.normalize_importance_weight(ps)
    path = tmp_path / "pmcsim"
    ps.write(path)
    back = pmcg.PmcSimu.read(path, N, D)
    old_logw = np.log(back.weights) + back.s.logSum
    # a second, independent likelihood: a broad Gaussian around the target's mean
    mu2 = mut[0] + 0.5
    second = pmcg.MixMvdens.from_arrays([1.0], mu2[None, :], cov=[np.eye(D) * 4.0], df=-1).cholesky()
    post2 = pmcg.Posterior(D).add_mix(second)
    count = back.importance_sample(post2)
    assert count == back.N
    om = oracle.Mix(np.array([1.0]), mu2[None, :], cov=np.eye(D)[None] * 4.0, df=-1)
    ref = oracle.mix_logpdf(om, back.X)
    np.testing.assert_allclose(back.weights, ref, rtol=1e-11, atol=1e-9)
    # combined log-weights and their normalisation
    comb = old_logw + back.weights
    back.weights[:] = comb
    back.host_modified()
    pmcg.normalize_importance_weight(back)
    m = comb.max()
    np.testing.assert_allclose(back.s.logSum, m + np.log(np.sum(np.exp(comb - m))), rtol=1e-10)


@pytest.mark.parametrize("D", [1, 6, 32, 64])
def test_weighted_moments_match_numpy(pmcg, D):
    rng = np.random.default_rng(D)
    N = 70001
    ps = pmcg.PmcSimu(N, D)
    X = rng.normal(0, 3, (N, D)) + rng.normal(0, 10, D)[None, :]
    logw = rng.normal(0, 2, N)
    flg = (rng.uniform(size=N) > 0.05).astype(np.int16)
    ps.X[:] = X
    ps.weights[:] = logw
    ps.flg[:] = flg
    ps.s.isLog = 1
    ps.host_modified()
    mean, cov = ps.weighted_moments()
    k = flg == 1
    wb = np.exp(logw[k] - logw[k].max())
    wb /= wb.sum()
    m_ref = wb @ X[k]
    d = X[k] - m_ref
    c_ref = (wb[:, None] * d).T @ d
    np.testing.assert_allclose(mean, m_ref, rtol=1e-9, atol=1e-9)
    sig = np.sqrt(np.diag(c_ref))
    assert np.max(np.abs(cov - c_ref) / np.outer(sig, sig)) < 1e-5
    np.testing.assert_array_equal(cov, cov.T)


@pytest.mark.parametrize("median", [False, True])
def test_weighted_summary_matches_oracle(pmcg, oracle, median):
    """Marginal centre and one-sided limits on the device (sort + FP64 scan)
    against the reference's sequential loops (oracle), on a sample with
    uncounted points and unequal weights."""
    rng = np.random.default_rng(31 + median)
    N, D = 50001, 5
    X = rng.normal(0, 2, (N, D)) + np.arange(D)[None, :]
    logw = rng.normal(0, 1.5, N)
    flg = (rng.uniform(size=N) > 0.1).astype(np.int16)
    ps = pmcg.PmcSimu(N, D)
    ps.X[:] = X
    ps.weights[:] = logw
    ps.flg[:] = flg
    ps.s.isLog = 1
    ps.host_modified()
    center, sigma = ps.weighted_summary(median=median)
    wbar, _, _ = oracle.normalize(logw, flg)
    c_ref, s_ref, st = oracle.weighted_summary(X, wbar, flg, median=median)
    assert np.all(st == 0)
    np.testing.assert_allclose(center, c_ref, rtol=1e-12, atol=1e-13)
    np.testing.assert_array_equal(sigma == -1.0, s_ref == -1.0)
    np.testing.assert_allclose(sigma, s_ref, rtol=1e-12, atol=1e-12)


def test_weighted_histograms_match_oracle(pmcg, oracle):
    rng = np.random.default_rng(5)
    N, D = 40003, 3
    X = rng.normal(0, 1, (N, D))
    X[:5, 0] = [-2.0, 2.0, -2.5, 2.5, 0.0]     # on the edges and outside
    logw = rng.normal(0, 1, N)
    flg = (rng.uniform(size=N) > 0.05).astype(np.int16)
    ps = pmcg.PmcSimu(N, D)
    ps.X[:] = X
    ps.weights[:] = logw
    ps.flg[:] = flg
    ps.s.isLog = 1
    ps.host_modified()
    lo, hi = np.array([-2.0, -3.0, -1.0]), np.array([2.0, 3.0, 1.0])
    wbar, _, _ = oracle.normalize(logw, flg)
    h = ps.weighted_hist1d(40, lo, hi)
    h_ref = oracle.hist1d(X, wbar, flg, 40, lo, hi, float(N))
    np.testing.assert_allclose(h, h_ref, rtol=1e-9, atol=1e-9)
    h2 = ps.weighted_hist2d(25, 0, 2, lo, hi)
    h2_ref = oracle.hist2d(X, wbar, flg, 25, 0, 2, lo, hi, float(N))
    np.testing.assert_allclose(h2, h2_ref, rtol=1e-9, atol=1e-9)


def test_fisher_matrix_of_a_gaussian_posterior(pmcg):
    """log P quadratic: the central differences give the precision matrix up to rounding;
    all stencil points in one batched device evaluation."""
    D = 5
    rng = np.random.default_rng(9)
    A = rng.normal(size=(D, D))
    cov = A @ A.T + np.eye(D)
    mu = rng.normal(size=D)
    lo, hi = mu - 20.0, mu + 20.0
    target = pmcg.MixMvdens.from_arrays([1.0], mu[None, :], cov=cov[None], df=-1).cholesky()
    post = pmcg.Posterior(D, lo, hi).add_mix(target)
    F = post.fisher(mu + 0.3, lo, hi)
    np.testing.assert_allclose(F, np.linalg.inv(cov), rtol=1e-6, atol=1e-8)
    np.testing.assert_array_equal(F, F.T)


def sn_fisher_oracle(oracle, sn, pos, lo, hi):
    """The reference's central differences (exec/go_fishing.c:37-86) on the
    oracle's FP64 SN log-likelihood (the flat prior cancels in the stencil)."""
    D = len(pos)
    h = 1e-3 * (hi - lo)
    sg = [(1, 1), (1, -1), (-1, 1), (-1, -1)]
    pts = []
    for a in range(D):
        for b in range(a + 1):
            for sa, sb in sg:
                x = pos.copy()
                x[a] += sa * h[a]
                x[b] += sb * h[b]
                pts.append(x)
    f, ok = oracle.sn_loglike(sn, np.array(pts))
    assert np.all(ok == 1)
    F = np.zeros((D, D))
    e = 0
    for a in range(D):
        for b in range(a + 1):
            v = f[4 * e:4 * e + 4]
            F[a, b] = F[b, a] = -(v[0] - v[1] - v[2] + v[3]) / (4 * h[a] * h[b])
            e += 1
    return F


def test_fisher_start_for_the_sn_posterior(pmcg, oracle):
    """SN posterior at the generating cosmology: the device Fisher matrix against the
    oracle's; the positiveness verdict; the diagonal-only and force-positive forms;
    an eigen-rule proposal from the latter inside the prior box."""
    wl = W.sn_workload()
    lo, hi = wl["bmin"], wl["bmax"]
    post = pmcg.Posterior(6, lo, hi).add_snia(wl["sn"])
    pos = W.SN_TRUTH.copy()
    F, pd = post.fisher(pos, lo, hi, with_positive=True)
    F_ref = sn_fisher_oracle(oracle, wl["sn"], pos, lo, hi)
    scale = np.sqrt(np.outer(np.abs(np.diag(F_ref)), np.abs(np.diag(F_ref))))
    assert np.max(np.abs(F - F_ref) / scale) < 1e-5
    np.testing.assert_array_equal(F, F.T)
    assert pd == bool(np.all(np.linalg.eigvalsh(F) > 0))
    Fd, pdd = post.fisher(pos, lo, hi, diag_only=True, with_positive=True)
    np.testing.assert_array_equal(np.diag(Fd), np.diag(F))
    assert np.count_nonzero(Fd - np.diag(np.diag(Fd))) == 0
    assert pdd == bool(np.all(np.diag(F) > 0))
    Fp, pdp = post.fisher(pos, lo, hi, force_positive=True, with_positive=True)
    np.testing.assert_array_equal(Fp, np.diag(np.abs(np.diag(F))))
    assert pdp
    prop = pmcg.fisher_proposal(pmcg.MixMvdens(10, 6), Fp, pos, lo, hi,
                                kind=pmcg.FISHER_EIGEN, fshift=0.1, fvar=1.0)
    _, mu, _ = prop.arrays()
    assert np.all(mu >= lo) and np.all(mu <= hi)


def test_max_posterior_of_a_gaussian(pmcg):
    """Nelder-Mead from three starts, advanced together (exec/max_post.c:182-224):
    every search ends at the mean, at the analytic maximum of log P."""
    D = 4
    rng = np.random.default_rng(12)
    A = rng.normal(size=(D, D))
    cov = A @ A.T + np.eye(D)
    mu = rng.normal(size=D)
    lo, hi = mu - 10.0, mu + 10.0
    target = pmcg.MixMvdens.from_arrays([1.0], mu[None, :], cov=cov[None], df=-1).cholesky()
    post = pmcg.Posterior(D, lo, hi).add_mix(target)
    starts = mu + rng.uniform(-3.0, 3.0, (3, D))
    x, lp, xs, lps = post.max_posterior(starts, lo, hi, ftol=1e-13)
    expected = -0.5 * D * np.log(2 * np.pi) - 0.5 * np.linalg.slogdet(cov)[1] - np.sum(np.log(hi - lo))
    sig = np.sqrt(np.diag(cov))
    assert lp == pytest.approx(expected, abs=1e-9)
    np.testing.assert_allclose(lps, expected, atol=1e-9)
    assert np.max(np.abs(xs - mu) / sig) < 1e-3


def test_max_posterior_evaluation_limit(pmcg):
    D = 3
    target = pmcg.MixMvdens.from_arrays([1.0], np.zeros((1, D)), cov=np.eye(D)[None], df=-1).cholesky()
    lo, hi = -np.ones(D) * 5, np.ones(D) * 5
    post = pmcg.Posterior(D, lo, hi).add_mix(target)
    with pytest.raises(pmcg.PmcgError) as e:
        post.max_posterior(np.full((1, D), 2.0), lo, hi, ftol=1e-14, max_evals=D + 3)
    assert e.value.code == -9012


def test_max_posterior_then_fisher_for_the_sn_posterior(pmcg, oracle):
    """The go_fishing start: maximum posterior from the generating cosmology and
    two nearby points, its log-likelihood against the oracle, and the diagonal
    Fisher matrix there (go_fishing's Fisher_diag remedy) positive definite:
    every parameter's own curvature is downward at the maximum. The full matrix
    can stay indefinite: SN data alone leave a nearly flat curved valley in
    (Omega_m, Omega_de, w0) whose curvature the central differences resolve to
    either sign."""
    wl = W.sn_workload()
    lo, hi = wl["bmin"], wl["bmax"]
    post = pmcg.Posterior(6, lo, hi).add_snia(wl["sn"])
    starts = np.stack([W.SN_TRUTH, W.SN_TRUTH + 0.02 * (hi - lo), W.SN_TRUTH - 0.02 * (hi - lo)])
    x, lp, _, _ = post.max_posterior(starts, lo, hi, ftol=1e-10)
    logpr = -np.sum(np.log(hi - lo))
    ll, ok = oracle.sn_loglike(wl["sn"], np.stack([x, W.SN_TRUTH]))
    assert ok.all()
    assert lp == pytest.approx(ll[0] + logpr, rel=1e-11, abs=1e-8)
    assert ll[0] >= ll[1]
    Fd, pdd = post.fisher(x, lo, hi, diag_only=True, with_positive=True)
    assert pdd and np.all(np.diag(Fd) > 0)


@pytest.mark.parametrize("normalised", [False, True])
def test_clip_weights_matches_oracle(pmcg, oracle, normalised):
    """The nclipw largest weights leave the sample (flags bit-exact against the
    oracle, ties to the lower index); a normalised sample is renormalised."""
    rng = np.random.default_rng(40 + normalised)
    N, D, k = 30001, 3, 25
    logw = np.round(rng.normal(0, 2, N) * 2) / 2   # many equal weights: ties at the k-th place
    logw[[10, 20, 30]] = logw.max() + 1.0
    flg = (rng.uniform(size=N) > 0.1).astype(np.int16)
    flg[20] = 0                              # the largest but not counted
    ps = pmcg.PmcSimu(N, D)
    ps.X[:] = rng.normal(size=(N, D))
    ps.weights[:] = logw
    ps.flg[:] = flg
    ps.s.isLog = 1
    ps.host_modified()
    if normalised:
        pmcg.normalize_importance_weight(ps)
    pmcg.clip_weights(ps, k)
    ref = oracle.clip_weights(logw, flg, k)
    kth = np.sort(logw[flg == 1])[::-1][k - 1]
    assert np.sum(logw[flg == 1] == kth) > 1          # the boundary is a tie
    np.testing.assert_array_equal(ps.flg, ref)
    assert np.sum(flg) - np.sum(ps.flg) == k
    if normalised:
        keep = ref == 1
        m = logw[keep].max()
        wb = np.exp(logw[keep] - m)
        wb /= wb.sum()
        np.testing.assert_allclose(ps.weights[keep], wb, rtol=1e-12)
        assert ps.s.logSum == pytest.approx(m + np.log(np.sum(np.exp(logw[keep] - m))), rel=1e-12)


def test_sample_file_read_with_clipping(pmcg, tmp_path):
    """pmc_simu_from_file with nclipw > 0 (the resumed run of
    exec/cosmo_pmc.c:416-417): the sample read back equals the same file read
    without clipping and then clipped with clip_weights."""
    rng = np.random.default_rng(12)
    N, D, k = 4000, 3, 7
    ps = pmcg.PmcSimu(N, D)
    ps.X[:] = rng.normal(size=(N, D))
    logw = rng.normal(size=N) * 2
    ps.weights[:] = np.exp(logw - logw.max()) / np.sum(np.exp(logw - logw.max()))
    ps.flg[:] = 1
    ps.indices[:] = rng.integers(0, 5, N)
    ps.s.isLog = 0
    ps.s.logSum = logw.max() + np.log(np.sum(np.exp(logw - logw.max())))
    path = tmp_path / "pmcsim"
    ps.write(path)
    a = pmcg.PmcSimu.read(path, N, D, nclipw=k)
    b = pmcg.PmcSimu.read(path, N, D)
    pmcg.clip_weights(b, k)
    np.testing.assert_array_equal(a.flg, b.flg)
    np.testing.assert_array_equal(a.weights, b.weights)
    assert a.s.logSum == b.s.logSum and a.s.nok == N - k
