"""Tensor-core (tcgen05, three-term TF32 split) mixture log-density against the
CUDA-core single-precision kernel and the FP64 oracle, through the C ABI.

Tolerances are those of the single-precision path: per-sample |d log q| below
5e-3 (max) and 5e-4 (mean) on the condition-1e6 D=32 Student-t mixture, 1e-3
on well-conditioned mixtures; whole iterations |d log Z| <= 1e-3 and posterior
means/covariances within 0.05 sigma of the FP64 path.
"""
import numpy as np
import pytest

from cosmopmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture
def tensor_cores(pmcg):
    prev = pmcg.set_tensor_cores(True)
    yield
    pmcg.set_tensor_cores(prev)


def make_mix(pmcg, w, mu, cov, df):
    return pmcg.MixMvdens.from_arrays(w, mu, cov=cov, df=df).cholesky()


def oracle_mix(oracle, m):
    w, mu, L = m.arrays()
    return oracle.Mix(w, mu, df=m.df, L=L)


def logpdf_both(pmcg, m, X):
    """(tensor-core, CUDA-core) single-precision log-densities and terms."""
    prev = pmcg.set_tensor_cores(True)
    try:
        tc = pmcg.mix_log_pdf_batch(m, X, precision=pmcg.MIXED, want_terms=True)
        pmcg.set_tensor_cores(False)
        cc = pmcg.mix_log_pdf_batch(m, X, precision=pmcg.MIXED, want_terms=True)
    finally:
        pmcg.set_tensor_cores(prev)
    return tc, cc


def test_switch_returns_previous_setting(pmcg):
    prev = pmcg.set_tensor_cores(True)
    assert pmcg.set_tensor_cores(False) == 1
    assert pmcg.set_tensor_cores(prev) == 0


@pytest.mark.parametrize("N", [1, 255, 257, 3000])
def test_condition_1e6_student_t(pmcg, oracle, N):
    """D=32, K=64, nu=3, covariance condition 1e6, points drawn from the mixture."""
    wl = W.mixture_workload(D=32, K=64, seed=5)
    w, mu, cov, df = wl["prop"]
    m = make_mix(pmcg, w, mu, cov, df)
    om = oracle_mix(oracle, m)
    u, z, chi2 = oracle.randoms(9, 0, N, 32, df)
    X, _, _, _ = oracle.draw(om, u, z, chi2)
    ref, lt_ref, _ = oracle.mix_logpdf(om, X, want_terms=True)
    (lq_tc, lt_tc), (lq_cc, lt_cc) = logpdf_both(pmcg, m, X)
    err = np.abs(lq_tc - ref)
    assert np.max(err) < 5e-3 and np.mean(err) < 5e-4, (np.max(err), np.mean(err))
    # per-component terms: same accuracy class as the CUDA-core kernel
    fin = np.isfinite(lt_ref)
    scale = np.maximum(1.0, np.abs(lt_ref[fin]))
    e_tc = np.abs(lt_tc[fin] - lt_ref[fin]) / scale
    e_cc = np.abs(lt_cc[fin] - lt_ref[fin]) / scale
    assert np.max(e_tc) < max(4 * np.max(e_cc), 1e-5), (np.max(e_tc), np.max(e_cc))
    if N >= 255:  # a different kernel ran: not bit-identical to the CUDA-core result
        assert not np.array_equal(lq_tc, lq_cc)


@pytest.mark.parametrize("shape", [(64, 32, -1), (5, 23, 3), (1, 17, -1), (13, 8, 5), (3, 1, -1), (6, 30, 4),
                                   (129, 20, -1)])
def test_shapes_against_oracle(pmcg, oracle, shape):
    """Odd K (padding components of the last group of 4), D below 32 (padding
    rows / columns), a single component, D = 1; K = 129 (an odd number of
    component groups) over more tiles than SMs, so that each CTA runs several
    tiles and the operand buffers alternate across tile boundaries."""
    K, D, df = shape
    rng = np.random.default_rng(K * 100 + D)
    mu = rng.normal(0, 2, (K, D))
    A = rng.normal(0, 1, (K, D, D))
    cov = np.einsum("kij,klj->kil", A, A) + np.eye(D)[None]
    w = rng.dirichlet(np.ones(K) * 3)
    m = make_mix(pmcg, w, mu, cov, df)
    om = oracle_mix(oracle, m)
    X = rng.normal(0, 3, (50001 if K > 64 else 1001, D))
    ref, lt_ref, _ = oracle.mix_logpdf(om, X, want_terms=True)
    (lq_tc, lt_tc), _ = logpdf_both(pmcg, m, X)
    np.testing.assert_allclose(lq_tc, ref, rtol=0, atol=1e-3 * max(1.0, np.max(np.abs(ref)) / 100))
    fin = np.isfinite(lt_ref)
    assert np.array_equal(np.isfinite(lt_tc), fin)
    np.testing.assert_allclose(lt_tc[fin], lt_ref[fin], rtol=1e-4, atol=1e-3)


def test_dead_component_terms(pmcg, oracle):
    """A zero-weight component contributes -inf terms and nothing to the sum."""
    K, D = 6, 24
    rng = np.random.default_rng(11)
    mu = rng.normal(0, 1, (K, D))
    cov = np.repeat(np.eye(D)[None], K, axis=0)
    w = np.full(K, 1.0 / (K - 1))
    w[2] = 0.0
    m = make_mix(pmcg, w, mu, cov, -1)
    om = oracle_mix(oracle, m)
    X = rng.normal(0, 1, (700, D))
    ref = oracle.mix_logpdf(om, X)
    (lq_tc, lt_tc), _ = logpdf_both(pmcg, m, X)
    np.testing.assert_allclose(lq_tc, ref, rtol=0, atol=1e-4)
    assert np.all(lt_tc[2] == -np.inf)


def weighted_moments(X, wbar):
    mean = wbar @ X
    d = X - mean
    return mean, (wbar[:, None] * d).T @ d


def test_run_meets_precision_targets(pmcg, tensor_cores):
    """Whole iterations of the D=32, K=64, nu=3 (condition 1e6) mixture workload
    with the tensor-core proposal and target densities against the FP64 path."""
    wl = W.mixture_workload(D=32, K=64, Kt=16, seed=64)
    w, mu, cov, df = wl["prop"]
    wt, mut, covt, _ = wl["target"]
    prop = make_mix(pmcg, w, mu, cov, df)
    target = make_mix(pmcg, wt, mut, covt, -1)
    post = pmcg.Posterior(32).add_mix(target)
    N = 65536
    r64 = pmcg.Run(prop, post, N, precision=0, seed=7)
    r32 = pmcg.Run(prop, post, N, precision=1, seed=7)
    for it in range(2):
        s64 = r64.iterate(1.0)
        s32 = r32.iterate(1.0)
        assert abs(s64["ln_evidence"] - s32["ln_evidence"]) <= 1e-3, (it, s64, s32)
        p64, p32 = r64.sample(), r32.sample()
        wb64 = np.where(p64.flg == 1, np.exp(p64.weights - s64["logSum"]), 0.0)
        wb32 = np.where(p32.flg == 1, np.exp(p32.weights - s32["logSum"]), 0.0)
        m64, c64 = weighted_moments(p64.X, wb64)
        m32, c32 = weighted_moments(p32.X, wb32)
        sig = np.sqrt(np.diag(c64))
        assert np.max(np.abs(m64 - m32) / sig) < 0.05
        assert np.max(np.abs(c64 - c32) / np.outer(sig, sig)) < 0.05
        w64, mu64, L64 = r64.proposal().arrays()
        w32, mu32, L32 = r32.proposal().arrays()
        live = (w64 > 0) & (w32 > 0)
        sd = np.sqrt(np.diagonal(np.einsum("kij,klj->kil", L64, L64), axis1=1, axis2=2))
        assert np.max(np.abs(mu64[live] - mu32[live]) / sd[live]) < 0.05
        assert np.max(np.abs(w64 - w32)) < 1e-3


# ----------------------------------------------------------------- template likelihood
def _tpl_both(pmcg, post, T):
    prev = pmcg.set_tensor_cores(True)
    try:
        tc = post.log_pdf_batch(T, precision=pmcg.MIXED)
        pmcg.set_tensor_cores(False)
        cc = post.log_pdf_batch(T, precision=pmcg.MIXED)
    finally:
        pmcg.set_tensor_cores(prev)
    return tc, cc


@pytest.mark.parametrize("N", [1, 77, 128, 129, 30001])
def test_template_tensor_cores_vs_oracle(pmcg, oracle, N):
    """c2 shape (D=12, P=91, M=2048): chi2 = |U phi|^2 on the tensor cores against
    the FP64 oracle: |d log L| < 5e-3 over the prior box (chi2 up to ~1e4;
    3e-6 relative) and < 2e-3 at the truth; ragged tiles (N not a multiple of
    128, fewer samples than one tile)."""
    wl = W.template_workload(D=12, M=2048)
    post = pmcg.Posterior(12).add_template(wl["A"], wl["C"], wl["dobs"])
    At, dt = oracle.tpl_prepare(wl["A"], wl["C"], wl["dobs"])
    T = np.random.default_rng(N).uniform(-1, 1, (N, 12))
    T[0] = wl["theta0"]
    ref = oracle.tpl_loglike(At, dt, T)
    (tc, ftc), (cc, fcc) = _tpl_both(pmcg, post, T)
    assert ftc.all() and fcc.all()
    err = np.abs(tc - ref)
    assert np.max(err) < 5e-3 and np.max(err / np.abs(ref)) < 3e-6, (np.max(err), np.max(err / np.abs(ref)))
    assert err[0] < 2e-3
    # the CUDA-core Gram form (its own tolerance, 1e-2) agrees too
    assert np.max(np.abs(cc - ref)) < 1e-2
    # every sample is computed alone: a prefix gives the same values bit for bit
    if N > 64:
        (tc_s, _), _ = _tpl_both(pmcg, post, T[:64])
        np.testing.assert_array_equal(tc_s, tc[:64])


@pytest.mark.parametrize("D", [1, 3, 7])
def test_template_tensor_cores_small_dimensions(pmcg, oracle, D):
    """P = 3, 10, 36 monomials (one to five K-steps; zero padding up to 96)."""
    wl = W.template_workload(D=D, M=257, seed=7 + D)
    post = pmcg.Posterior(D).add_template(wl["A"], wl["C"], wl["dobs"])
    At, dt = oracle.tpl_prepare(wl["A"], wl["C"], wl["dobs"])
    T = np.random.default_rng(D).uniform(-1, 1, (1000, D))
    ref = oracle.tpl_loglike(At, dt, T)
    (tc, _), _ = _tpl_both(pmcg, post, T)
    np.testing.assert_allclose(tc, ref, rtol=3e-6, atol=1e-3)


def test_template_tensor_cores_iteration_and_flags(pmcg):
    """A whole c2-shape iteration with the tensor-core template: the same ln Z as the
    CUDA-core run within 1e-3, and samples outside the box (flg = 0) skipped."""
    wl = W.template_workload(D=12, M=2048, K=16)
    F = W.template_fisher(wl)
    w, mu, cov, df = W.fisher_proposal(np.random.default_rng(3), 16, wl["theta0"], F, wl["bmin"], wl["bmax"])
    prop = make_mix(pmcg, w, mu, cov, df)
    post = pmcg.Posterior(12, wl["bmin"], wl["bmax"]).add_template(wl["A"], wl["C"], wl["dobs"])
    box = pmcg.Parabox(wl["bmin"], wl["bmax"])
    out = {}
    for on in (1, 0):
        prev = pmcg.set_tensor_cores(bool(on))
        try:
            run = pmcg.Run(prop, post, 100003, precision=pmcg.MIXED, seed=5, box=box)
            out[on] = [run.iterate(1.0) for _ in range(2)]
            s = run.sample()
            assert np.all(np.isneginf(s.weights[s.flg == 0]))
            run.free()
        finally:
            pmcg.set_tensor_cores(prev)
    for a, b in zip(out[1], out[0]):
        assert abs(a["ln_evidence"] - b["ln_evidence"]) < 1e-3, (a, b)
