"""pmcg_importance_weights_noalloc: the entry point for callers that cannot let
the library allocate device memory (code inside another framework's memory
pool, serving loops where an allocation would synchronise the device). Its
partial sums live in a fixed device array inside the library, so it must give
the same log-weights and evidence/perplexity/ESS as the allocating weight step
(generic_get_importance_weight_and_deduced_verb), call after call.

This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(pmcg):
    rng = np.random.default_rng(21)
    K, D = 5, 4
    mu = rng.normal(0, 2, (K, D))
    A = rng.normal(0, 1, (K, D, D))
    cov = np.einsum("kij,klj->kil", A, A) + np.eye(D)[None]
    prop = pmcg.MixMvdens.from_arrays(rng.dirichlet(np.ones(K) * 2), mu, cov=cov, df=4).cholesky()
    target = pmcg.MixMvdens.from_arrays([0.6, 0.4], mu[:2] + 0.3, cov=cov[:2] * 0.5, df=-1).cholesky()
    bmin, bmax = np.full(D, -7.0), np.full(D, 7.0)
    post = pmcg.Posterior(D, bmin, bmax).add_mix(target)
    return prop, post, pmcg.Parabox(bmin, bmax)


def test_noalloc_weights_match_allocating_entry_point(pmcg):
    torch = pytest.importorskip("torch")
    assert pmcg.device_count() > 0
    pmcg.set_dropin_precision(pmcg.FP64)
    prop, post, pb = _problem(pmcg)
    N, beta = 100003, 0.9
    ps = pmcg.PmcSimu(N, prop.D)
    pmcg.simulate_mix_mvdens(ps, prop, pmcg.Rng(5), pb)
    X, flg0 = ps.X.copy(), ps.flg.copy()
    # the existing (allocating) entry point
    pmcg.importance_weights(ps, prop, post, beta)
    logw_ref, flg_ref = ps.weights.copy(), ps.flg.copy()
    perp_ref, ess_ref = pmcg.perplexity_and_ess(ps)
    _, lnz_ref = pmcg.evidence(ps)
    logsum_ref, maxw_ref = ps.s.logSum, ps.s.maxW
    # inputs of the new entry point, on the device (FP64 kernels of the library)
    logq = pmcg.mix_log_pdf_batch(prop, X, precision=pmcg.FP64)
    logpost, _ = post.log_pdf_batch(X, precision=pmcg.FP64)
    dev = torch.device("cuda", 0)
    lp_d = torch.tensor(logpost, dtype=torch.float64, device=dev)
    lq_d = torch.tensor(logq, dtype=torch.float64, device=dev)
    lib = pmcg.load()
    for call in range(2):
        flg_d = torch.tensor(flg0, dtype=torch.int16, device=dev)
        logw_d = torch.full((N,), 7.0, dtype=torch.float64, device=dev)
        st = pmcg.WeightStats()
        err = pmcg._Err()
        torch.cuda.synchronize()
        lib.pmcg_importance_weights_noalloc(N, beta, lp_d.data_ptr(), lq_d.data_ptr(), flg_d.data_ptr(),
                                            logw_d.data_ptr(), C.byref(st), None, err.ref)
        err.check()
        torch.cuda.synchronize()
        logw = logw_d.cpu().numpy()
        flg = flg_d.cpu().numpy()
        np.testing.assert_array_equal(flg, flg_ref)
        ok = flg == 1
        np.testing.assert_allclose(logw[ok], logw_ref[ok], rtol=1e-12, atol=1e-9)
        assert np.all(np.isneginf(logw[~ok]))
        assert abs(st.logSum - logsum_ref) < 1e-10
        assert st.maxW == maxw_ref
        assert abs(st.ln_evidence - lnz_ref) < 1e-10
        assert abs(st.perplexity / perp_ref - 1.0) < 1e-10
        assert abs(st.ess / ess_ref - 1.0) < 1e-10
        assert st.nok == int(ok.sum())


def test_noalloc_rejects_more_samples_than_its_scratch_holds(pmcg):
    torch = pytest.importorskip("torch")
    lib = pmcg.load()
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    f = torch.ones(8, dtype=torch.int16, device="cuda")
    st = pmcg.WeightStats()
    err = pmcg._Err()
    lib.pmcg_importance_weights_noalloc(8388609, 1.0, t.data_ptr(), t.data_ptr(), f.data_ptr(), t.data_ptr(),
                                        C.byref(st), None, err.ref)
    with pytest.raises(pmcg.PmcgError) as e:
        err.check()
    assert e.value.code == -9002


def _call(pmcg, lib, N, beta, lp_d, lq_d, flg_d, logw_d):
    st = pmcg.WeightStats()
    err = pmcg._Err()
    lib.pmcg_importance_weights_noalloc(N, beta, lp_d.data_ptr(), lq_d.data_ptr(), flg_d.data_ptr(),
                                        logw_d.data_ptr(), C.byref(st), None, err.ref)
    return st, err


def test_noalloc_at_its_sample_limit_matches_a_float64_reduction(pmcg):
    """N = 8,388,608 exactly (4096 partial records, the merge's strided loop at its
    longest), some samples flagged out, against numpy in float64."""
    torch = pytest.importorskip("torch")
    lib = pmcg.load()
    N, beta = 8388608, 0.7
    rng = np.random.default_rng(8)
    lp = rng.normal(-3.0, 2.0, N)
    lq = rng.normal(0.0, 1.5, N)
    flg = (rng.uniform(size=N) > 0.05).astype(np.int16)
    dev = torch.device("cuda", 0)
    lp_d = torch.tensor(lp, device=dev)
    lq_d = torch.tensor(lq, device=dev)
    for call in range(2):
        flg_d = torch.tensor(flg, device=dev)
        logw_d = torch.zeros(N, dtype=torch.float64, device=dev)
        st, err = _call(pmcg, lib, N, beta, lp_d, lq_d, flg_d, logw_d)
        err.check()
        ok = flg == 1
        l = beta * lp[ok] - lq[ok]
        m = l.max()
        s = np.exp(l - m).sum()
        logsum = m + np.log(s)
        wb = np.exp(l - logsum)
        assert abs(st.logSum - logsum) < 1e-9
        assert st.maxW == m
        assert abs(st.ln_evidence - (logsum - np.log(N))) < 1e-9
        perp = np.exp(-np.sum(wb * np.log(wb))) / N
        assert abs(st.perplexity / perp - 1.0) < 1e-9
        assert abs(st.ess / (1.0 / np.sum(wb * wb)) - 1.0) < 1e-9
        assert st.nok == int(ok.sum())
        logw = logw_d.cpu().numpy()
        np.testing.assert_allclose(logw[ok], l, rtol=1e-12, atol=1e-12)  # FMA contraction on the device
        assert np.all(np.isneginf(logw[~ok]))


def test_noalloc_reports_no_weight_when_every_sample_is_flagged_out(pmcg):
    torch = pytest.importorskip("torch")
    lib = pmcg.load()
    N = 5000
    t = torch.zeros(N, dtype=torch.float64, device="cuda")
    flg_d = torch.zeros(N, dtype=torch.int16, device="cuda")
    logw_d = torch.zeros(N, dtype=torch.float64, device="cuda")
    st, err = _call(pmcg, lib, N, 1.0, t, t, flg_d, logw_d)
    with pytest.raises(pmcg.PmcgError) as e:
        err.check()
    assert e.value.code == -9011
    assert np.all(np.isneginf(logw_d.cpu().numpy()))
