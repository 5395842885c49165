"""The FP64 oracle against the golden fixtures (scipy / numpy restatements,
published Philox vectors, reference demo targets). CPU only."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
G = np.load(os.path.join(GOLD, "golden.npz"))
META = json.load(open(os.path.join(GOLD, "golden.json")))


def test_philox_known_answers(oracle):
    for c, k, o in zip(G["philox_ctr"], G["philox_key"], G["philox_out"]):
        assert oracle.philox([int(v) for v in c], [int(v) for v in k]) == [int(v) for v in o]


@pytest.mark.parametrize("tag", ["gauss", "t"])
def test_mixture_logpdf_vs_scipy(oracle, tag):
    m = oracle.Mix(G[f"mix_{tag}_w"], G[f"mix_{tag}_mu"], G[f"mix_{tag}_cov"], df=META[f"mix_{tag}_df"])
    lq = oracle.mix_logpdf(m, G[f"mix_{tag}_X"])
    np.testing.assert_allclose(lq, G[f"mix_{tag}_logq"], rtol=0, atol=1e-11)


def test_lum_dist_vs_quad(oracle):
    for c, row in zip(G["dl_cosmo"], G["dl_val"]):
        for z, ref in zip(G["dl_z"], row):
            d, st = oracle.lum_dist(*c, z, G=8, nsub=32)
            assert st == 1
            assert abs(d / ref - 1) < 1e-12


@pytest.mark.parametrize("tag", ["full", "marg", "logdet"])
def test_sn_loglike_vs_reference(oracle, tag):
    sn = dict(META[f"sn_{tag}"])
    for k in ("z", "mB", "x1", "c", "cov6"):
        sn[k] = G[f"sn_{tag}_{k}"]
    ll, ok = oracle.sn_loglike(sn, G[f"sn_{tag}_P"])
    assert ok.all()
    np.testing.assert_allclose(ll, G[f"sn_{tag}_ll"], rtol=1e-11, atol=1e-9)


def test_sn_loitering_is_flagged(oracle):
    sn = dict(META["sn_full"])
    for k in ("z", "mB", "x1", "c", "cov6"):
        sn[k] = G[f"sn_full_{k}"]
    # Omega_m = 0, Omega_de = 1.5, w0 = -3: E^2 < 0 at moderate z
    ll, ok = oracle.sn_loglike(sn, np.array([[0.0, 1.5, -3.0, -19.1, 0.1, 3.0]]))
    assert ok[0] == 0


def test_template_loglike_vs_numpy(oracle):
    At, dt = oracle.tpl_prepare(G["tpl_A"], G["tpl_C"], G["tpl_dobs"])
    ll = oracle.tpl_loglike(At, dt, G["tpl_T"])
    np.testing.assert_allclose(ll, G["tpl_ll"], rtol=1e-10)


def test_weights_evidence_perplexity(oracle):
    flg = G["wt_flg"].astype(np.int16)
    lw = oracle.logweights(META["wt_beta"], G["wt_lp"], G["wt_lq"], flg)
    wbar, ls, mw = oracle.normalize(lw, flg)
    perp, ess = oracle.perplexity(wbar, flg)
    ls_ref, mw_ref, perp_ref, ess_ref, lnz_ref = G["wt_expect"]
    assert abs(ls - ls_ref) < 1e-12 and mw == mw_ref
    assert abs(perp / perp_ref - 1) < 1e-12 and abs(ess / ess_ref - 1) < 1e-12
    assert abs((ls - np.log(len(flg))) - lnz_ref) < 1e-12


@pytest.mark.parametrize("tag", ["gauss", "t"])
def test_em_update_vs_numpy(oracle, tag):
    df = META[f"em_{tag}_df"]
    m = oracle.Mix(G[f"em_{tag}_w"], G[f"em_{tag}_mu"], G[f"em_{tag}_cov"], df=df)
    X = G[f"em_{tag}_X"]
    flg = G[f"em_{tag}_flg"].astype(np.int16)
    logq, lt, Q = oracle.mix_logpdf(m, X, want_terms=True)
    new, dead = oracle.update_rb(m, X, G[f"em_{tag}_wbar"], flg, lt, logq, Q, G[f"em_{tag}_idx"])
    np.testing.assert_array_equal(dead, G[f"em_{tag}_dead"])
    np.testing.assert_allclose(new.w, G[f"em_{tag}_nw"], rtol=1e-11, atol=1e-15)
    live = dead == 0
    np.testing.assert_allclose(new.mu[live], G[f"em_{tag}_nmu"][live], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(new.cov[live], G[f"em_{tag}_ncov"][live], rtol=1e-10, atol=1e-12)


def test_tempering_schedule(oracle):
    for kind, it, b in G["tempering"]:
        assert abs(oracle.tempering_beta(int(kind), int(it), 0.05, 6) - b) < 1e-15


def test_draw_indices_and_transform(oracle):
    rng = np.random.default_rng(5)
    K, D = 5, 3
    w = rng.dirichlet(np.ones(K))
    mu = rng.normal(size=(K, D))
    cov = np.array([np.eye(D) * (k + 1) for k in range(K)])
    m = oracle.Mix(w, mu, cov, df=-1)
    u, z, chi2 = oracle.randoms(7, 0, 20000, D, 0)
    X, idx, flg, nok = oracle.draw(m, u, z, chi2)
    cw = np.cumsum(w)
    ref = np.array([np.argmax(uu < cw) if uu < cw[-1] else K - 1 for uu in u])
    np.testing.assert_array_equal(idx, ref)
    np.testing.assert_allclose(X, mu[idx] + np.einsum("nij,nj->ni", m.L[idx], z), rtol=1e-13, atol=1e-13)
    # component frequencies and normal moments are right
    assert np.all(np.abs(np.bincount(idx, minlength=K) / len(u) - w) < 0.02)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02
    assert nok == len(u)


def test_chi2_variates_have_nu_mean(oracle):
    u, z, chi2 = oracle.randoms(3, 1, 20000, 5, 3)
    assert abs(chi2.mean() - 3.0) < 0.1
    assert abs(chi2.var() - 6.0) < 0.5


@pytest.mark.skipif("demo1_mean" not in G.files, reason="reference demo targets not captured")
def test_demo_targets_give_unit_evidence(oracle):
    """Full oracle PMC on the two tempering demos: evidence ~ 1 (analytic)."""
    for tag, K in (("demo1", 3), ("demo2", 6)):
        mean, cov = G[f"{tag}_mean"], G[f"{tag}_cov"]
        Kt = len(mean)
        target = oracle.Mix(np.full(Kt, 1.0 / Kt), mean, cov, df=-1)
        rng = np.random.default_rng(2)
        prop = oracle.Mix(np.full(K, 1.0 / K), rng.uniform(0.2, 0.8, (K, 2)), np.array([np.eye(2) * 0.05] * K))
        bmin, bmax = np.zeros(2), np.ones(2)
        for it in range(8):
            st = oracle.iterate_mix(prop, target, 0.0, 20000, 99, it, bmin=bmin, bmax=bmax)
        assert abs(np.exp(st["ln_evidence"]) - META["demo_analytic_evidence"]) < 0.02, st
