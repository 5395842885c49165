"""The oracle's posterior-composition terms (posterior_log_pdf_common,
wrappers/src/param.c:958-1041) on the CPU: the special prior's constant
(prior_log_pdf_special, :1055-1101) against the formulas written out here, and
the subset prior (config prior with indprior, :1009-1026) against scipy."""
import numpy as np
import pytest
from scipy import stats

BMIN = np.array([0.0, 0.0, -3.0, -1.5, -20.0])
BMAX = np.array([1.2, 1.5, 0.0, 1.0, -18.5])


def test_special_none_and_unity(oracle):
    assert oracle.prior_special(0, BMIN, BMAX) == 0.0
    # unity cancels the flat prior -sum log(max - min)
    assert abs(oracle.prior_special(1, BMIN, BMAX) - np.sum(np.log(BMAX - BMIN))) < 1e-15


def test_special_de_conservative(oracle):
    c = oracle.prior_special(2, BMIN, BMAX, ind_w0=2)
    assert abs(c - (np.log(3.0) - np.log(2.0 / 3.0))) < 1e-15
    a_acc = 0.6
    t = 0.5 * (2.0 / 3.0) ** 2
    c2 = oracle.prior_special(2, BMIN, BMAX, ind_w0=2, ind_w1=3, a_acc=a_acc)
    assert abs(c2 - (np.log(3.0) + np.log(2.5) - np.log(t / (1 - a_acc)) - np.log(t))) < 1e-14
    # no w0 among the parameters: nothing added
    assert oracle.prior_special(2, BMIN, BMAX, ind_w0=-1) == 0.0
    # a w0 range narrower than [-1, -1/3] is an error
    with pytest.raises(ValueError):
        oracle.prior_special(2, BMIN, np.where(np.arange(5) == 2, -0.5, BMAX), ind_w0=2)


@pytest.mark.parametrize("df", [-1, 5])
def test_subset_prior_vs_scipy(oracle, df):
    rng = np.random.default_rng(3)
    X = rng.normal(0, 1, (400, 6))
    ind = np.array([0, 1, 0, 1, 1, 0])
    mean = np.array([0.2, -0.3, 0.5])
    A = rng.normal(0, 1, (3, 3))
    cov = A @ A.T + 0.5 * np.eye(3)
    got = oracle.mvdens_prior_logpdf(mean, cov, df, X, ind)
    sub = X[:, ind == 1]
    ref = (stats.multivariate_normal(mean, cov).logpdf(sub) if df <= 0
           else stats.multivariate_t(mean, cov, df=df).logpdf(sub))
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11)
    # indprior None: every parameter
    full = oracle.mvdens_prior_logpdf(np.zeros(6), np.eye(6), -1, X)
    np.testing.assert_allclose(full, stats.multivariate_normal(np.zeros(6), np.eye(6)).logpdf(X), atol=1e-11)
