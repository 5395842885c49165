"""CUDA path vs the FP64 oracle and the golden fixtures, through the C ABI.

Tolerances: the FP64 path must agree with the oracle to rounding (stated per
test, 1e-9..1e-12). The mixed path (FP32 quadratic forms / likelihoods with
FP64 reductions) must give |d log Z| <= 1e-3 and posterior means/covariances
within 0.05 sigma; per-sample log-densities are checked at the stated looser
absolute tolerances.
"""
import json
import os

import numpy as np
import pytest

from cosmopmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
G = np.load(os.path.join(GOLD, "golden.npz"))
META = json.load(open(os.path.join(GOLD, "golden.json")))

PRECS = [0, 1]


@pytest.fixture(scope="module", autouse=True)
def _gpu(pmcg):
    assert pmcg.device_count() > 0, "no CUDA device visible"


def make_mix(pmcg, w, mu, cov, df):
    return pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()


def oracle_mix(oracle, m):
    w, mu, L = m.arrays()
    return oracle.Mix(w, mu, df=m.df, L=L)


def small_mixture(K=7, D=5, df=-1, seed=3):
    rng = np.random.default_rng(seed)
    mu = rng.normal(0, 2, (K, D))
    A = rng.normal(0, 1, (K, D, D))
    cov = np.einsum("kij,klj->kil", A, A) + np.eye(D)[None]
    w = rng.dirichlet(np.ones(K) * 3)
    return w, mu, cov, df


# ----------------------------------------------------------------- (a) draws
@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", [(7, 5, -1), (7, 5, 3), (64, 32, 3), (1, 1, -1), (3, 7, 5)])
def test_draw_indices_bit_exact(pmcg, oracle, prec, shape):
    K, D, df = shape
    w, mu, cov, _ = small_mixture(K, D, df)
    m = make_mix(pmcg, w, mu, cov, df)
    N = 5003
    pmcg.set_dropin_precision(prec)
    ps = pmcg.PmcSimu(N, D)
    rng = pmcg.Rng(1234)
    bmin, bmax = mu.min(0) - 1.0, mu.max(0) + 1.0
    pb = pmcg.Parabox(bmin, bmax)
    nok = pmcg.simulate_mix_mvdens(ps, m, rng, pb)
    om = oracle_mix(oracle, m)
    u, z, chi2 = oracle.randoms(1234, 0, N, D, df)
    X, idx, flg, nok_o = oracle.draw(om, u, z, chi2, bmin, bmax)
    np.testing.assert_array_equal(ps.indices, idx)
    if prec == 0:
        np.testing.assert_allclose(ps.X, X, rtol=1e-12, atol=1e-12)
        np.testing.assert_array_equal(ps.flg, flg)
        assert nok == nok_o
    else:
        # single-precision transform: error relative to |x| (a Student-t draw with a
        # small chi^2 lands far out) plus the component scale
        scale = np.sqrt(np.max(np.diagonal(cov, axis1=1, axis2=2))) + np.abs(mu).max()
        assert np.max(np.abs(ps.X - X) / (np.abs(X) + scale)) < 2e-6
        assert np.sum(ps.flg != flg) <= 2
    assert rng.calls == 1


def test_dropin_ranged_draw_equals_single_pass(pmcg, oracle):
    """The single-precision drop-in draw runs in sample ranges whose host copies
    overlap the next range's draw: the sample equals the engine's single-pass
    draw of the same seed bit for bit, indices equal the oracle's (N not a
    multiple of the range count, a box that rejects some samples)."""
    K, D, df = 64, 32, 3
    w, mu, cov, _ = small_mixture(K, D, df, seed=12)
    m = make_mix(pmcg, w, mu, cov, df)
    N = 100003
    bmin, bmax = mu.min(0) - 30.0, mu.max(0) + 30.0   # rejects part of the Student-t tails
    pmcg.set_dropin_precision(1)
    ps = pmcg.PmcSimu(N, D)
    rng = pmcg.Rng(4321)
    nok = pmcg.simulate_mix_mvdens(ps, m, rng, pmcg.Parabox(bmin, bmax))
    run = pmcg.Run(m, pmcg.Posterior(D, bmin, bmax).add_mix(m), N, precision=1, seed=4321,
                   box=pmcg.Parabox(bmin, bmax))
    run.iterate(1.0)
    ref = run.sample()
    np.testing.assert_array_equal(ps.X, ref.X)
    np.testing.assert_array_equal(ps.indices, ref.indices)
    np.testing.assert_array_equal(ps.flg, ref.flg)
    assert nok == int(np.sum(ps.flg != 0)) and 0 < nok < N
    om = oracle_mix(oracle, m)
    u, z, chi2 = oracle.randoms(4321, 0, N, D, df)
    _, idx, _, _ = oracle.draw(om, u, z, chi2, bmin, bmax)
    np.testing.assert_array_equal(ps.indices, idx)
    run.free()


def test_sn_large_sample_against_oracle(pmcg, oracle):
    """Single precision over 40000 random points of the prior box (several waves
    of one warp per point) against the FP64 oracle; a 3000-point subset alone
    gives the same values."""
    wl = W.sn_workload()
    sn = wl["sn"]
    post = pmcg.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(sn)
    rng = np.random.default_rng(41)
    N = 40000
    P = rng.uniform(wl["bmin"], wl["bmax"], (N, 6))
    ref, ok = oracle.sn_loglike(sn, P)
    ref = ref + (-np.sum(np.log(wl["bmax"] - wl["bmin"])))
    ll, flg = post.log_pdf_batch(P, precision=1)
    ll_s, flg_s = post.log_pdf_batch(P[:3000], precision=1)
    good = ok == 1
    assert np.sum((flg == 1) != good) <= 2
    np.testing.assert_array_equal(flg_s, flg[:3000])
    np.testing.assert_array_equal(ll_s, ll[:3000])
    # relative error grows with chi^2 (FP32 integrand nodes): 1e-4 over 40000 box points
    b = good & (flg == 1)
    assert np.max(np.abs(ll[b] - ref[b]) / np.maximum(1.0, np.abs(ref[b]))) < 1e-4


# ----------------------------------------------------------------- (b) mixture log-pdf
@pytest.mark.parametrize("tag", ["gauss", "t"])
def test_mix_logpdf_golden(pmcg, tag):
    m = make_mix(pmcg, G[f"mix_{tag}_w"], G[f"mix_{tag}_mu"], G[f"mix_{tag}_cov"], META[f"mix_{tag}_df"])
    lq = pmcg.mix_log_pdf_batch(m, G[f"mix_{tag}_X"], precision=0)
    np.testing.assert_allclose(lq, G[f"mix_{tag}_logq"], rtol=0, atol=1e-10)
    lq32 = pmcg.mix_log_pdf_batch(m, G[f"mix_{tag}_X"], precision=1)
    np.testing.assert_allclose(lq32, G[f"mix_{tag}_logq"], rtol=0, atol=2e-4)


def test_mix_logpdf_condition_1e6(pmcg, oracle):
    """D=32, K=64 Student-t nu=3 with covariance condition 1e6, points drawn from it."""
    wl = W.mixture_workload(D=32, K=64, seed=5)
    w, mu, cov, df = wl["prop"]
    m = make_mix(pmcg, w, mu, cov, df)
    om = oracle_mix(oracle, m)
    u, z, chi2 = oracle.randoms(9, 0, 3000, 32, df)
    X, idx, flg, _ = oracle.draw(om, u, z, chi2)
    ref, lt_ref, _ = oracle.mix_logpdf(om, X, want_terms=True)
    lq, lt = pmcg.mix_log_pdf_batch(m, X, precision=0, want_terms=True)
    np.testing.assert_allclose(lq, ref, rtol=0, atol=1e-9)
    np.testing.assert_allclose(lt, lt_ref, rtol=1e-12, atol=1e-8)
    lq32 = pmcg.mix_log_pdf_batch(m, X, precision=1)
    err = np.abs(lq32 - ref)
    assert np.max(err) < 5e-3 and np.mean(err) < 5e-4, (np.max(err), np.mean(err))


# ----------------------------------------------------------------- (c) likelihoods
@pytest.mark.parametrize("tag", ["full", "marg", "logdet"])
def test_sn_loglike_golden(pmcg, tag):
    sn = dict(META[f"sn_{tag}"])
    for k in ("z", "mB", "x1", "c", "cov6"):
        sn[k] = G[f"sn_{tag}_{k}"]
    post = pmcg.Posterior(6).add_snia(sn)
    ll, flg = post.log_pdf_batch(G[f"sn_{tag}_P"], precision=0)
    assert flg.all()
    np.testing.assert_allclose(ll, G[f"sn_{tag}_ll"], rtol=1e-11, atol=1e-8)
    ll32, flg32 = post.log_pdf_batch(G[f"sn_{tag}_P"], precision=1)
    assert flg32.all()
    np.testing.assert_allclose(ll32, G[f"sn_{tag}_ll"], rtol=0, atol=2e-3)


def test_sn_740_vs_oracle_and_loitering(pmcg, oracle):
    wl = W.sn_workload()
    sn = wl["sn"]
    post = pmcg.Posterior(6, wl["bmin"], wl["bmax"]).add_snia(sn)
    rng = np.random.default_rng(4)
    P = rng.uniform(wl["bmin"], wl["bmax"], (701, 6))
    P[0] = [0.0, 1.5, -3.0, -19.1, 0.1, 3.0]   # loitering: E^2 < 0
    ref, ok = oracle.sn_loglike(sn, P)
    ll, flg = post.log_pdf_batch(P, precision=0)
    np.testing.assert_array_equal(flg, ok)
    logpr = -np.sum(np.log(wl["bmax"] - wl["bmin"]))
    good = ok == 1
    assert flg[0] == 0
    np.testing.assert_allclose(ll[good], ref[good] + logpr, rtol=1e-11, atol=1e-8)
    ll32, flg32 = post.log_pdf_batch(P, precision=1)
    both = good & (flg32 == 1)
    assert np.sum(flg32 != ok) <= 2
    # FP32 integrand nodes: the error grows with chi^2 (relative 3e-5 far from the truth) ...
    assert np.max(np.abs(ll32[both] - ll[both]) / np.maximum(1.0, np.abs(ll[both]))) < 3e-5
    # ... and stays below 2e-3 absolute near the truth (chi^2 ~ N_SN)
    truth = np.array([0.3, 0.7, -1.0, -19.1, 0.14, 3.1])[None, :]
    l64, _ = post.log_pdf_batch(truth, precision=0)
    l32, _ = post.log_pdf_batch(truth, precision=1)
    assert abs(l64[0] - l32[0]) < 2e-3


def test_template_golden_and_c2_shape(pmcg, oracle):
    post = pmcg.Posterior(3).add_template(G["tpl_A"], G["tpl_C"], G["tpl_dobs"])
    ll, flg = post.log_pdf_batch(G["tpl_T"], precision=0)
    np.testing.assert_allclose(ll, G["tpl_ll"], rtol=1e-10)
    ll32, _ = post.log_pdf_batch(G["tpl_T"], precision=1)
    np.testing.assert_allclose(ll32, G["tpl_ll"], rtol=0, atol=1e-3)
    wl = W.template_workload(D=12, M=2048)
    post2 = pmcg.Posterior(12).add_template(wl["A"], wl["C"], wl["dobs"])
    At, dt = oracle.tpl_prepare(wl["A"], wl["C"], wl["dobs"])
    T = np.random.default_rng(1).uniform(-1, 1, (300, 12))
    T[0] = wl["theta0"]
    ref = oracle.tpl_loglike(At, dt, T)
    ll, _ = post2.log_pdf_batch(T, precision=0)
    np.testing.assert_allclose(ll, ref, rtol=1e-11)
    ll32, _ = post2.log_pdf_batch(T, precision=1)
    assert np.max(np.abs(ll32 - ref)) < 1e-2
    assert np.max(np.abs(ll32[:1] - ref[:1])) < 1e-3  # near the best fit (chi2 ~ 2048)


# ----------------------------------------------------------------- (d)+(e) drop-in sequence
def dropin_iteration(pmcg, m, post, N, seed, beta, box, prec):
    pmcg.set_dropin_precision(prec)
    ps = pmcg.PmcSimu(N, m.D)
    rng = pmcg.Rng(seed)
    pb = pmcg.Parabox(*box) if box is not None else None
    pmcg.simulate_mix_mvdens(ps, m, rng, pb)
    nok = pmcg.importance_weights(ps, m, post, beta)
    logw = ps.weights.copy()
    ls = pmcg.normalize_importance_weight(ps)
    wbar = ps.weights.copy()
    perp, ess = pmcg.perplexity_and_ess(ps)
    ev, lnev = pmcg.evidence(ps)
    X, idx, flg = ps.X.copy(), ps.indices.copy(), ps.flg.copy()
    pmcg.update_prop_rb(m, ps)
    return dict(ps=ps, nok=nok, logw=logw, logSum=ls, wbar=wbar, perp=perp, ess=ess, lnev=lnev, X=X, idx=idx,
                flg=flg)


@pytest.mark.parametrize("df", [-1, 4])
def test_dropin_iteration_fp64_matches_oracle(pmcg, oracle, df):
    w, mu, cov, _ = small_mixture(K=6, D=4, df=df, seed=8)
    wt, mut, covt, _ = small_mixture(K=3, D=4, df=-1, seed=9)
    m = make_mix(pmcg, w, mu, cov, df)
    om = oracle_mix(oracle, m)
    target = make_mix(pmcg, wt, mut, covt, -1)
    ot = oracle_mix(oracle, target)
    bmin, bmax = np.full(4, -6.0), np.full(4, 6.0)
    post = pmcg.Posterior(4, bmin, bmax).add_mix(target)
    N, beta = 20011, 0.8
    r = dropin_iteration(pmcg, m, post, N, 77, beta, (bmin, bmax), 0)
    # oracle on the device sample
    X, flg = r["X"], r["flg"].astype(np.int16)
    logq, lt, Q = oracle.mix_logpdf(om, X, want_terms=True)
    lp = oracle.mix_logpdf(ot, X) - np.sum(np.log(bmax - bmin))
    lw = oracle.logweights(beta, lp, logq, flg)
    np.testing.assert_allclose(r["logw"][flg == 1], lw[flg == 1], rtol=1e-12, atol=1e-9)
    assert np.all(np.isneginf(r["logw"][flg == 0]))
    wbar, ls, mw = oracle.normalize(lw, flg)
    assert abs(r["logSum"] - ls) < 1e-10
    np.testing.assert_allclose(r["wbar"], wbar, rtol=1e-9, atol=1e-15)
    perp, ess = oracle.perplexity(wbar, flg)
    assert abs(r["perp"] / perp - 1) < 1e-10 and abs(r["ess"] / ess - 1) < 1e-10
    assert abs(r["lnev"] - (ls - np.log(N))) < 1e-10
    new, dead = oracle.update_rb(om, X, wbar, flg, lt, logq, Q, r["idx"])
    w2, mu2, L2 = m.arrays()
    np.testing.assert_allclose(w2, new.w, rtol=1e-9, atol=1e-14)
    live = dead == 0
    np.testing.assert_allclose(mu2[live], new.mu[live], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(L2[live], new.L[live], rtol=1e-8, atol=1e-11)


@pytest.mark.parametrize("prec", PRECS)
def test_dropin_lookahead_hit_and_miss(pmcg, prec):
    """simulate_mix_mvdens evaluates log q, and the log-posterior of the posterior the
    previous weight step used, while X travels to the host; the weight step keeps
    what matches its arguments. Results equal those of a fresh sample object (no
    look-ahead) holding the same draw, both when the posterior is the same (hit) and
    when it changes (miss: the SN posterior's look-ahead flagged loitering
    cosmologies, and the draw's own flags come back before the other posterior)."""
    wl = W.sn_workload(K=10, init="fisher")
    w, mu, cov, _ = wl["prop"]
    # plus a component around a loitering cosmology (Omega_m ~ 0.05, Omega_de ~ 1.4, w0 ~ -2.8)
    loiter = np.array([0.05, 1.4, -2.8, -19.1, 0.14, 3.1])
    w2 = np.append(w * 0.5, 0.5)
    mu2 = np.vstack([mu, loiter[None, :]])
    cov2 = np.concatenate([cov, np.diag([0.02, 0.05, 0.1, 0.05, 0.02, 0.2])[None] ** 2 * 4.0])
    m = make_mix(pmcg, w2, mu2, cov2, -1)
    bmin, bmax = wl["bmin"], wl["bmax"]
    post_a = pmcg.Posterior(6, bmin, bmax).add_snia(wl["sn"])
    wt = np.array([1.0])
    post_b = pmcg.Posterior(6, bmin, bmax).add_mix(make_mix(pmcg, wt, mu[:1], cov[:1] * 4.0, -1))
    pmcg.set_dropin_precision(prec)
    N = 20000
    pb = pmcg.Parabox(bmin, bmax)

    def fresh(call, post):
        ps = pmcg.PmcSimu(N, 6)
        rng = pmcg.Rng(5)
        rng.p.contents.calls = call
        pmcg.simulate_mix_mvdens(ps, m, rng, pb)
        nok = pmcg.importance_weights(ps, m, post, 1.0)
        return nok, ps.weights.copy(), ps.flg.copy(), ps.X.copy()

    ps = pmcg.PmcSimu(N, 6)
    rng = pmcg.Rng(5)
    pmcg.simulate_mix_mvdens(ps, m, rng, pb)
    pmcg.importance_weights(ps, m, post_a, 1.0)        # remembers post_a
    for call, post in ((1, post_a), (2, post_b)):      # hit, then miss
        pmcg.simulate_mix_mvdens(ps, m, rng, pb)
        nok = pmcg.importance_weights(ps, m, post, 1.0)
        r_nok, r_w, r_f, r_x = fresh(call, post)
        np.testing.assert_array_equal(ps.X, r_x)
        np.testing.assert_array_equal(ps.flg, r_f)
        np.testing.assert_array_equal(ps.weights, r_w)
        assert nok == r_nok
    # the miss case really had a look-ahead to undo: the SN posterior flags some of these points
    _, _, f_a, _ = fresh(2, post_a)
    assert np.sum(f_a == 0) > np.sum(ps.flg == 0)


@pytest.mark.parametrize("tag", ["gauss", "t"])
def test_update_prop_rb_golden(pmcg, tag):
    """update_prop_rb on a host-built sample (normalised weights) vs the numpy EM."""
    pmcg.set_dropin_precision(0)
    df = META[f"em_{tag}_df"]
    m = make_mix(pmcg, G[f"em_{tag}_w"], G[f"em_{tag}_mu"], G[f"em_{tag}_cov"], df)
    X = G[f"em_{tag}_X"]
    N, D = X.shape
    ps = pmcg.PmcSimu(N, D)
    ps.X[:] = X
    ps.flg[:] = G[f"em_{tag}_flg"]
    ps.indices[:] = G[f"em_{tag}_idx"]
    ps.weights[:] = G[f"em_{tag}_wbar"]
    ps.s.isLog = 0
    ps.host_modified()
    pmcg.update_prop_rb(m, ps)
    w, mu, L = m.arrays()
    dead = G[f"em_{tag}_dead"]
    np.testing.assert_allclose(w, G[f"em_{tag}_nw"], rtol=1e-10, atol=1e-15)
    live = dead == 0
    np.testing.assert_allclose(mu[live], G[f"em_{tag}_nmu"][live], rtol=1e-9, atol=1e-12)
    cov = np.einsum("kij,klj->kil", L, L)
    np.testing.assert_allclose(cov[live], G[f"em_{tag}_ncov"][live], rtol=1e-9, atol=1e-12)
    assert w[dead == 1].sum() == 0.0


# ----------------------------------------------------------------- full runs
def c1_small(pmcg, N, D=32, K=64, Kt=16):
    wl = W.mixture_workload(D=D, K=K, Kt=Kt, seed=64)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = make_mix(pmcg, w, mu, cov, df)
    target = make_mix(pmcg, wt, mut, covt, -1)
    post = pmcg.Posterior(D).add_mix(target)
    return prop, target, post


def test_run_fp64_matches_oracle_three_iterations(pmcg, oracle):
    prop, target, post = c1_small(pmcg, 0, D=12, K=16, Kt=4)
    op = oracle_mix(oracle, prop)
    ot = oracle_mix(oracle, target)
    N = 30000
    run = pmcg.Run(prop, post, N, precision=0, seed=42)
    for it in range(3):
        st = run.iterate(1.0)
        so = oracle.iterate_mix(op, ot, 0.0, N, 42, it)
        for key in ("ln_evidence", "perplexity", "ess", "enc", "logSum", "maxW"):
            assert abs(st[key] - so[key]) <= 1e-8 * max(1.0, abs(so[key])), (it, key, st[key], so[key])
        assert st["nok"] == so["nok"] and st["ndead"] == so["ndead"]
        w, mu, L = run.proposal().arrays()
        np.testing.assert_allclose(w, op.w, rtol=1e-8, atol=1e-13)
        np.testing.assert_allclose(mu, op.mu, rtol=1e-8, atol=1e-9)
        np.testing.assert_allclose(L, op.L, rtol=1e-7, atol=1e-9)
        # continue both from the device proposal so that rounding cannot accumulate
        op = oracle.Mix(w, mu, df=op.df, L=L)


def weighted_moments(X, wbar):
    m = wbar @ X
    d = X - m
    return m, (wbar[:, None] * d).T @ d


def test_run_mixed_meets_precision_targets(pmcg, oracle):
    """c1 shape (D=32, K=64, nu=3, condition 1e6) at reduced N: |dlogZ| <= 1e-3 and
    posterior mean/covariance within 0.05 sigma of the FP64 path on the same draws."""
    prop, target, post = c1_small(pmcg, 0)
    N = 65536
    r64 = pmcg.Run(prop, post, N, precision=0, seed=7)
    r32 = pmcg.Run(prop, post, N, precision=1, seed=7)
    for it in range(2):
        s64 = r64.iterate(1.0)
        s32 = r32.iterate(1.0)
        assert abs(s64["ln_evidence"] - s32["ln_evidence"]) <= 1e-3, (it, s64, s32)
        p64, p32 = r64.sample(), r32.sample()
        if it == 0:  # same proposal: bit-exact; after one update the weights differ by rounding
            np.testing.assert_array_equal(p64.indices, p32.indices)
        else:
            assert np.mean(p64.indices != p32.indices) < 1e-3
        wb64 = np.where(p64.flg == 1, np.exp(p64.weights - s64["logSum"]), 0.0)
        wb32 = np.where(p32.flg == 1, np.exp(p32.weights - s32["logSum"]), 0.0)
        m64, c64 = weighted_moments(p64.X, wb64)
        m32, c32 = weighted_moments(p32.X, wb32)
        sig = np.sqrt(np.diag(c64))
        assert np.max(np.abs(m64 - m32) / sig) < 0.05
        assert np.max(np.abs(c64 - c32) / np.outer(sig, sig)) < 0.05
        # updated proposals agree too
        w64, mu64, L64 = r64.proposal().arrays()
        w32, mu32, L32 = r32.proposal().arrays()
        live = (w64 > 0) & (w32 > 0)
        sd = np.sqrt(np.diagonal(np.einsum("kij,klj->kil", L64, L64), axis1=1, axis2=2))
        assert np.max(np.abs(mu64[live] - mu32[live]) / sd[live]) < 0.05
        assert np.max(np.abs(w64 - w32)) < 1e-3


def test_evidence_known_answer_normalised_target(pmcg):
    """No prior box, normalised Gaussian-mixture target: log Z = 0."""
    prop, target, post = c1_small(pmcg, 0, D=6, K=8, Kt=3)
    run = pmcg.Run(prop, post, 200000, precision=1, seed=3)
    for it in range(6):
        st = run.iterate(1.0)
    assert abs(st["ln_evidence"]) < 0.02, st
    assert st["perplexity"] > 0.5


@pytest.mark.skipif("demo1_mean" not in G.files, reason="reference demo targets not captured")
@pytest.mark.parametrize("prec", PRECS)
def test_reference_tempering_demos_unit_evidence(pmcg, prec):
    """Demo/tempering 1 and 2 (unit box, normalised targets): evidence = 1."""
    for tag, K in (("demo1", 3), ("demo2", 6)):
        mean, cov = G[f"{tag}_mean"], G[f"{tag}_cov"]
        target = make_mix(pmcg, np.full(len(mean), 1.0 / len(mean)), mean, cov, -1)
        rng = np.random.default_rng(2)
        prop = make_mix(pmcg, np.full(K, 1.0 / K), rng.uniform(0.2, 0.8, (K, 2)), np.array([np.eye(2) * 0.05] * K),
                        -1)
        bmin, bmax = np.zeros(2), np.ones(2)
        post = pmcg.Posterior(2, bmin, bmax).add_mix(target)
        run = pmcg.Run(prop, post, 20000, precision=prec, seed=11, box=pmcg.Parabox(bmin, bmax))
        for it in range(8):
            st = run.iterate(1.0)
        assert abs(np.exp(st["ln_evidence"]) - 1.0) < 0.02, (tag, st)


# ----------------------------------------------------------------- edge cases
def test_all_samples_outside_box_raises(pmcg):
    pmcg.set_dropin_precision(0)
    m = make_mix(pmcg, [1.0], [[10.0, 10.0]], [np.eye(2) * 0.01], -1)
    target = make_mix(pmcg, [1.0], [[0.0, 0.0]], [np.eye(2)], -1)
    post = pmcg.Posterior(2, [-1, -1], [1, 1]).add_mix(target)
    ps = pmcg.PmcSimu(257, 2)
    nok = pmcg.simulate_mix_mvdens(ps, m, pmcg.Rng(1), pmcg.Parabox([-1, -1], [1, 1]))
    assert nok == 0
    with pytest.raises(pmcg.PmcgError) as e:
        pmcg.importance_weights(ps, m, post, 1.0)
    assert e.value.code == -9011


def test_dead_component_is_buried(pmcg):
    w = np.array([0.999, 0.001])
    m = make_mix(pmcg, w, [[0.0, 0.0], [3.0, 3.0]], [np.eye(2), np.eye(2)], -1)
    target = make_mix(pmcg, [1.0], [[0.0, 0.0]], [np.eye(2)], -1)
    post = pmcg.Posterior(2).add_mix(target)
    for prec in PRECS:
        run = pmcg.Run(m, post, 5000, precision=prec, seed=5)
        st = run.iterate(1.0)
        w2, _, _ = run.proposal().arrays()
        assert w2[1] == 0.0 and abs(w2[0] - 1.0) < 1e-15 and st["ndead"] == 1
        assert abs(st["enc"] - 1.0) < 1e-12


@pytest.mark.parametrize("N", [1, 31, 129, 4097])
def test_ragged_sample_counts(pmcg, oracle, N):
    w, mu, cov, _ = small_mixture(K=3, D=3)
    m = make_mix(pmcg, w, mu, cov, -1)
    om = oracle_mix(oracle, m)
    X = np.random.default_rng(N).normal(size=(N, 3))
    for prec, tol in ((0, 1e-10), (1, 1e-3)):
        lq = pmcg.mix_log_pdf_batch(m, X, precision=prec)
        np.testing.assert_allclose(lq, oracle.mix_logpdf(om, X), atol=tol, rtol=0)


def test_runs_are_bit_reproducible(pmcg):
    prop, target, post = c1_small(pmcg, 0, D=8, K=10, Kt=3)
    out = []
    for rep in range(2):
        run = pmcg.Run(prop, post, 50000, precision=1, seed=9)
        out.append([tuple(sorted(run.iterate(1.0).items())) for _ in range(2)])
    assert out[0] == out[1]


def test_tempered_weights(pmcg, oracle):
    """beta multiplies the log-posterior only (log w = beta log pi - log q)."""
    w, mu, cov, _ = small_mixture(K=3, D=2, seed=12)
    m = make_mix(pmcg, w, mu, cov, -1)
    target = make_mix(pmcg, [1.0], [[0.0, 0.0]], [np.eye(2)], -1)
    post = pmcg.Posterior(2, [-10, -10], [10, 10]).add_mix(target)
    r = dropin_iteration(pmcg, m, post, 4000, 5, 0.25, None, 0)
    om = oracle_mix(oracle, make_mix(pmcg, w, mu, cov, -1))
    X = r["X"]
    lw = 0.25 * (oracle.mix_logpdf(oracle_mix(oracle, target), X) - np.log(400.0)) - oracle.mix_logpdf(om, X)
    np.testing.assert_allclose(r["logw"], lw, rtol=1e-12, atol=1e-10)


def test_dropin_speculation_equals_fresh_sequence(pmcg):
    """Single precision, sample copied in ranges: after the draw the weight step
    (for the beta of the last two weight steps), the normalisation and the EM
    update run ahead while X travels to the host, and the calls that follow use
    them when their arguments match. Every iteration of the pmclib sequence must
    equal the same iteration on a fresh sample object (no history, nothing run
    ahead) bit for bit: hits (repeated beta), beta misses, a posterior change and
    a clip between the normalisation and the update."""
    P = pmcg
    wl = W.mixture_workload(D=8, K=4, Kt=2, nu=5, seed=17, prop_hi=2.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    target = make_mix(P, wt, mut, covt, -1)
    post_a = P.Posterior(8).add_mix(target)
    post_b = P.Posterior(8).add_mix(make_mix(P, wt[:1] / wt[0], mut[:1], covt[:1] * 2.0, -1))
    P.set_dropin_precision(P.MIXED)
    N = 40000   # eight draw ranges of at least 4096 samples
    m = make_mix(P, w, mu, cov, df)
    ps = P.PmcSimu(N, 8)
    rng = P.Rng(23)
    steps = [(1.0, post_a, 0), (1.0, post_a, 0), (1.0, post_a, 0), (1.0, post_a, 0), (0.5, post_a, 0),
             (0.5, post_a, 0), (0.5, post_a, 0), (1.0, post_a, 0), (1.0, post_a, 0), (1.0, post_b, 0),
             (1.0, post_b, 0), (1.0, post_b, 25), (1.0, post_b, 0)]
    try:
        for it, (beta, post, nclip) in enumerate(steps):
            wa, mua, La = m.arrays()
            mf = P.MixMvdens.from_arrays(wa, mua, L=La, df=m.df)
            out = []
            for mm, sim, r in ((m, ps, rng), (mf, P.PmcSimu(N, 8), P.Rng(23))):
                r.p.contents.calls = it
                P.simulate_mix_mvdens(sim, mm, r, None)
                nok = P.importance_weights(sim, mm, post, beta)
                lw = sim.weights.copy()
                ls = P.normalize_importance_weight(sim)
                if nclip:
                    P.clip_weights(sim, nclip)
                wb = sim.weights.copy()
                P.update_prop_rb(mm, sim)
                out.append((nok, lw, ls, wb, sim.flg.copy(), sim.X.copy(), P.perplexity_and_ess(sim),
                            P.evidence(sim), mm.arrays()))
            a, b = out
            assert a[0] == b[0] and a[2] == b[2], it
            for i in (1, 3, 4, 5):
                np.testing.assert_array_equal(a[i], b[i], err_msg=f"iteration {it} field {i}")
            assert a[6] == b[6] and a[7] == b[7], it
            for x, y in zip(a[8], b[8]):
                np.testing.assert_array_equal(x, y, err_msg=f"iteration {it} proposal")
    finally:
        P.set_dropin_precision(P.FP64)


def test_dropin_precision_per_sample(pmcg):
    """pmcg_simu_set_precision: with the process default single precision, a
    sample set to FP64 gives what a sample under the FP64 default gives, bit
    for bit, while another sample in the same process stays single precision."""
    P = pmcg
    wl = W.mixture_workload(D=6, K=3, Kt=2, nu=-1, seed=31, prop_hi=2.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    post = P.Posterior(6).add_mix(make_mix(P, wt, mut, covt, -1))
    N = 5000

    def one(sim, prec=None):
        m = make_mix(P, w, mu, cov, df)
        if prec is not None:
            sim.set_precision(prec)
        r = P.Rng(5)
        P.simulate_mix_mvdens(sim, m, r, None)
        P.importance_weights(sim, m, post, 1.0)
        ls = P.normalize_importance_weight(sim)
        P.update_prop_rb(m, sim)
        return sim.X.copy(), sim.weights.copy(), ls, m.arrays()

    try:
        P.set_dropin_precision(P.FP64)
        ref64 = one(P.PmcSimu(N, 6))
        P.set_dropin_precision(P.MIXED)
        ref32 = one(P.PmcSimu(N, 6))
        a = one(P.PmcSimu(N, 6), P.FP64)
        b = one(P.PmcSimu(N, 6))
        for x, y in ((a, ref64), (b, ref32)):
            np.testing.assert_array_equal(x[0], y[0])
            np.testing.assert_array_equal(x[1], y[1])
            assert x[2] == y[2]
            for u, v in zip(x[3], y[3]):
                np.testing.assert_array_equal(u, v)
        assert not np.array_equal(a[1], b[1])
        with pytest.raises(P.PmcgError):
            P.PmcSimu(N, 6).set_precision(7)
    finally:
        P.set_dropin_precision(P.FP64)


@pytest.mark.parametrize("D", [40, 64])
def test_run_mixed_beyond_the_tensor_cores(pmcg, D):
    """Single precision for 32 < D <= 64 (CUDA-core log-density, the whitened EM
    with its larger shared-memory layout): whole iterations against the FP64
    path on the same draws, |dlogZ| <= 1e-3 and the updated means within
    0.05 sigma."""
    P = pmcg
    wl = W.mixture_workload(D=D, K=4, Kt=2, nu=5, seed=D, prop_hi=2.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = make_mix(P, w, mu, cov, df)
    post = P.Posterior(D).add_mix(make_mix(P, wt, mut, covt, -1))
    r64 = P.Run(prop, post, 60000, precision=P.FP64, seed=9)
    r32 = P.Run(prop, post, 60000, precision=P.MIXED, seed=9)
    for it in range(3):
        s64, s32 = r64.iterate(1.0), r32.iterate(1.0)
        assert abs(s64["ln_evidence"] - s32["ln_evidence"]) <= 1e-3, (it, s64, s32)
        w64, mu64, L64 = r64.proposal().arrays()
        w32, mu32, L32 = r32.proposal().arrays()
        live = (w64 > 0) & (w32 > 0)
        sd = np.sqrt(np.diagonal(np.einsum("kij,klj->kil", L64, L64), axis1=1, axis2=2))
        assert np.max(np.abs(mu64[live] - mu32[live]) / sd[live]) < 0.05, it
    r64.free()
    r32.free()


def test_run_mixed_at_the_largest_component_count(pmcg):
    """K = 256 components (the largest supported; 32 tensor-core component
    groups): whole iterations of the mixed path against the FP64 path on the
    same draws, |dlogZ| <= 1e-3."""
    P = pmcg
    D, K = 8, 256
    wl = W.mixture_workload(D=D, K=K, Kt=8, nu=4, seed=256, prop_hi=1.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = make_mix(P, w, mu, cov, df)
    post = P.Posterior(D).add_mix(make_mix(P, wt, mut, covt, -1))
    r64 = P.Run(prop, post, 200000, precision=P.FP64, seed=4)
    r32 = P.Run(prop, post, 200000, precision=P.MIXED, seed=4)
    for it in range(2):
        s64, s32 = r64.iterate(1.0), r32.iterate(1.0)
        assert abs(s64["ln_evidence"] - s32["ln_evidence"]) <= 1e-3, (it, s64, s32)
        assert abs(s64["ess"] - s32["ess"]) <= 1e-3 * s64["ess"], (it, s64, s32)
    r64.free()
    r32.free()


@pytest.mark.parametrize("N", [1, 33, 257])
def test_run_tiny_and_ragged_sample_sizes(pmcg, N):
    """N below and just above one tensor-core tile of 256 samples: the mixed path
    (tensor cores on) and the FP64 path on the same draws either both fail with
    the same code (too few samples: every component buried) or agree on ln Z to
    1e-3 and on the draws' component indices."""
    P = pmcg
    wl = W.mixture_workload(D=12, K=4, Kt=2, nu=3, seed=N, prop_hi=1.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = make_mix(P, w, mu, cov, df)
    post = P.Posterior(12).add_mix(make_mix(P, wt, mut, covt, -1))
    prev = P.set_tensor_cores(True)
    try:
        r64 = P.Run(prop, post, N, precision=P.FP64, seed=N)
        r32 = P.Run(prop, post, N, precision=P.MIXED, seed=N)
        out = []
        for r in (r64, r32):
            try:
                out.append(("ok", r.iterate(1.0), r.sample().indices.copy()))
            except P.PmcgError as e:
                out.append(("err", e.code, None))
        (k64, a64, i64), (k32, a32, i32) = out
        assert k64 == k32, (N, out)
        if k64 == "err":
            assert a64 == a32
        else:
            assert abs(a64["ln_evidence"] - a32["ln_evidence"]) <= 1e-3, (N, a64, a32)
            np.testing.assert_array_equal(i64, i32)
        r64.free()
        r32.free()
    finally:
        P.set_tensor_cores(prev)


@pytest.mark.parametrize("prec", [0, 1])
def test_dropin_final_iteration_with_a_larger_sample(pmcg, prec):
    """The reference driver reallocates the sample for its last iteration
    (nsamples x fsfinal, exec/cosmo_pmc.c:300-320): after iterations at N, the
    iteration at 2N on the reallocated sample equals the same iteration on a
    fresh sample of 2N from the same proposal and generator state."""
    P = pmcg
    wl = W.mixture_workload(D=6, K=3, Kt=2, nu=-1, seed=71, prop_hi=1.0)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    post = P.Posterior(6).add_mix(make_mix(P, wt, mut, covt, -1))
    N = 30000
    try:
        P.set_dropin_precision(prec)
        m = make_mix(P, w, mu, cov, df)
        ps = P.PmcSimu(N, 6)
        rng = P.Rng(19)
        for it in range(3):
            rng.p.contents.calls = it
            P.simulate_mix_mvdens(ps, m, rng, None)
            P.importance_weights(ps, m, post, 1.0)
            P.normalize_importance_weight(ps)
            P.update_prop_rb(m, ps)
        wa, mua, La = m.arrays()
        P.call("pmc_simu_realloc", ps.p, 2 * N)
        fresh = P.PmcSimu(2 * N, 6)
        out = []
        for sim, mm in ((ps, m), (fresh, P.MixMvdens.from_arrays(wa, mua, L=La, df=m.df))):
            r = P.Rng(19)
            r.p.contents.calls = 3
            P.simulate_mix_mvdens(sim, mm, r, None)
            nok = P.importance_weights(sim, mm, post, 1.0)
            ls = P.normalize_importance_weight(sim)
            P.update_prop_rb(mm, sim)
            out.append((nok, ls, sim.X.copy(), sim.weights.copy(), mm.arrays()))
        a, b = out
        assert a[0] == b[0] and a[1] == b[1]
        np.testing.assert_array_equal(a[2], b[2])
        np.testing.assert_array_equal(a[3], b[3])
        for x, y in zip(a[4], b[4]):
            np.testing.assert_array_equal(x, y)
    finally:
        P.set_dropin_precision(P.FP64)
