"""ctypes bindings of the FP64 C oracle (oracle/pmc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py, as the reference the CUDA path is compared with. The
product library never imports
it. Parity with pmclib/nicaea is unpinned (both are external, absent
libraries); the oracle is pinned to scipy and analytic answers by
tests/golden.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libpmc_oracle.so")
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_sp = np.ctypeslib.ndpointer(dtype=np.int16, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "pmc_oracle.c")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB


class SN(C.Structure):
    _fields_ = [
        ("nsn", C.c_int),
        ("z", C.c_void_p), ("mB", C.c_void_p), ("x1", C.c_void_p), ("c", C.c_void_p),
        ("cov6", C.c_void_p),
        ("sig_int", C.c_double), ("v_pec", C.c_double), ("h", C.c_double),
        ("chi2mode", C.c_int), ("add_logdet", C.c_int), ("quad_nodes", C.c_int),
        ("ip_om", C.c_int), ("ip_ode", C.c_int), ("ip_w0", C.c_int), ("ip_M", C.c_int),
        ("ip_alpha", C.c_int), ("ip_beta", C.c_int),
        ("def_om", C.c_double), ("def_w0", C.c_double), ("def_M", C.c_double),
        ("def_alpha", C.c_double), ("def_beta", C.c_double),
        ("neg_M", C.c_int), ("neg_beta", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [("ln_evidence", C.c_double), ("perplexity", C.c_double), ("ess", C.c_double),
                ("enc", C.c_double), ("logSum", C.c_double), ("maxW", C.c_double),
                ("nok", C.c_size_t), ("ndead", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.orc_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_randoms.argtypes = [C.c_uint64, C.c_uint32, C.c_size_t, C.c_size_t, C.c_int, C.c_int,
                                  _dp, _dp, _dp]
        L.orc_cholesky.argtypes = [C.c_int, _dp, _dp, C.POINTER(C.c_double)]
        L.orc_cholesky.restype = C.c_int
        L.orc_cumweights.argtypes = [C.c_int, _dp, _dp]
        L.orc_draw.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_size_t, _dp, _dp, _dp,
                               C.c_void_p, C.c_void_p, _dp, _ip, _sp]
        L.orc_draw.restype = C.c_size_t
        L.orc_mix_logpdf.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_size_t, _dp,
                                     C.c_void_p, _dp, C.c_void_p, C.c_void_p]
        L.orc_gauss_legendre.argtypes = [C.c_int, _dp, _dp]
        L.orc_sn_loglike.argtypes = [C.POINTER(SN), C.c_size_t, C.c_int, _dp, C.c_void_p, _dp, C.c_void_p]
        L.orc_sn_loglike_one.argtypes = [C.POINTER(SN), _dp, C.POINTER(C.c_int)]
        L.orc_sn_loglike_one.restype = C.c_double
        L.orc_lum_dist.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                   C.c_int, C.POINTER(C.c_int)]
        L.orc_lum_dist.restype = C.c_double
        L.orc_tpl_prepare.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_tpl_prepare.restype = C.c_int
        L.orc_tpl_loglike.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_size_t, _dp, C.c_void_p, _dp]
        L.orc_logweights.argtypes = [C.c_size_t, C.c_double, _dp, _dp, _sp, _dp]
        L.orc_normalize.argtypes = [C.c_size_t, _dp, _sp, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_normalize.restype = C.c_int
        L.orc_perplexity.argtypes = [C.c_size_t, _dp, _sp, C.POINTER(C.c_double)]
        L.orc_perplexity.restype = C.c_double
        L.orc_enc.argtypes = [C.c_int, _dp]
        L.orc_enc.restype = C.c_double
        L.orc_tempering_beta.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int]
        L.orc_tempering_beta.restype = C.c_double
        L.orc_update_rb.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int, C.c_size_t,
                                    _dp, _dp, _sp, _dp, _dp, C.c_void_p, _ip, _ip]
        L.orc_update_rb.restype = C.c_int
        L.orc_iterate_mix.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp,
                                      C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_double,
                                      C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint64, C.c_uint32,
                                      C.c_double, C.POINTER(Stats), C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_iterate_mix.restype = C.c_int
        L.orc_num_threads.restype = C.c_int
        L.orc_prior_special.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, C.c_int, C.c_double,
                                        C.POINTER(C.c_double)]
        L.orc_prior_special.restype = C.c_int
        L.orc_revive.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_uint64,
                                 C.c_uint32]
        L.orc_revive.restype = C.c_int
        L.orc_weighted_summary.argtypes = [C.c_size_t, C.c_int, _dp, _dp, _sp, C.c_int, _dp, _dp, _ip]
        L.orc_hist1d.argtypes = [C.c_size_t, C.c_int, _dp, _dp, _sp, C.c_int, _dp, _dp, C.c_double, _dp]
        L.orc_hist2d.argtypes = [C.c_size_t, C.c_int, _dp, _dp, _sp, C.c_int, C.c_int, C.c_int, _dp, _dp,
                                 C.c_double, _dp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- helpers
def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def randoms(seed, call, N, D, nu, n0=0):
    u = np.empty(N)
    z = np.empty((N, D))
    chi2 = np.empty(N)
    lib().orc_randoms(seed, call, n0, N, D, nu, u, z, chi2)
    return u, z, chi2


def cholesky(Cm):
    Cm = np.ascontiguousarray(Cm, dtype=np.float64)
    D = Cm.shape[0]
    L = np.empty_like(Cm)
    ld = C.c_double()
    rc = lib().orc_cholesky(D, Cm, L, C.byref(ld))
    if rc:
        raise ValueError("not positive definite")
    return L, ld.value


class Mix:
    """Mixture in oracle layout: w[K], mu[K,D], L[K,D,D] lower Cholesky, logdetL[K]."""

    def __init__(self, w, mu, cov=None, df=-1, L=None):
        self.w = np.ascontiguousarray(w, dtype=np.float64).copy()
        self.mu = np.ascontiguousarray(mu, dtype=np.float64).copy()
        self.K, self.D = self.mu.shape
        self.df = int(df)
        if L is None:
            Ls, lds = [], []
            for k in range(self.K):
                Lk, ld = cholesky(cov[k])
                Ls.append(Lk)
                lds.append(ld)
            self.L = np.ascontiguousarray(np.array(Ls))
            self.logdetL = np.array(lds)
        else:
            self.L = np.ascontiguousarray(L, dtype=np.float64).copy()
            self.logdetL = np.array([np.sum(np.log(np.diag(Lk))) for Lk in self.L])

    def copy(self):
        return Mix(self.w, self.mu, df=self.df, L=self.L)

    @property
    def cov(self):
        return np.einsum("kij,klj->kil", self.L, self.L)


def cumweights(w):
    cw = np.empty_like(w)
    lib().orc_cumweights(len(w), np.ascontiguousarray(w), cw)
    return cw


def draw(mix: Mix, u, z, chi2, bmin=None, bmax=None):
    N = len(u)
    X = np.empty((N, mix.D))
    idx = np.empty(N, dtype=np.int32)
    flg = np.empty(N, dtype=np.int16)
    cw = cumweights(mix.w)
    bmin_a = None if bmin is None else np.ascontiguousarray(bmin, dtype=np.float64)
    bmax_a = None if bmax is None else np.ascontiguousarray(bmax, dtype=np.float64)
    nok = lib().orc_draw(mix.K, mix.D, mix.df, cw, mix.w, mix.mu, mix.L, N,
                         np.ascontiguousarray(u), np.ascontiguousarray(z), np.ascontiguousarray(chi2),
                         _ptr(bmin_a), _ptr(bmax_a), X, idx, flg)
    return X, idx, flg, nok


def mix_logpdf(mix: Mix, X, want_terms=False):
    X = np.ascontiguousarray(X, dtype=np.float64)
    N = X.shape[0]
    logq = np.empty(N)
    lt = np.empty((mix.K, N)) if want_terms else None
    Q = np.empty((mix.K, N)) if want_terms else None
    lib().orc_mix_logpdf(mix.K, mix.D, mix.df, mix.w, mix.mu, mix.L, mix.logdetL, N, X, None,
                         logq, _ptr(lt), _ptr(Q))
    return (logq, lt, Q) if want_terms else logq


def gauss_legendre(G):
    x = np.empty(G)
    w = np.empty(G)
    lib().orc_gauss_legendre(G, x, w)
    return x, w


def make_sn(data: dict, keep):
    """Build an SN struct from a dict of numpy arrays; `keep` holds the arrays alive."""
    s = SN()
    arrs = {k: np.ascontiguousarray(data[k], dtype=np.float64) for k in ("z", "mB", "x1", "c", "cov6")}
    keep.append(arrs)
    s.nsn = len(arrs["z"])
    for k, a in arrs.items():
        setattr(s, k, a.ctypes.data)
    for k in ("sig_int", "v_pec", "h", "def_om", "def_w0", "def_M", "def_alpha", "def_beta"):
        setattr(s, k, float(data[k]))
    for k in ("chi2mode", "add_logdet", "quad_nodes", "ip_om", "ip_ode", "ip_w0", "ip_M", "ip_alpha", "ip_beta"):
        setattr(s, k, int(data[k]))
    s.neg_M, s.neg_beta = int(data.get("neg_M", 0)), int(data.get("neg_beta", 0))
    return s


def sn_loglike(data: dict, X, flg=None):
    keep = []
    s = make_sn(data, keep)
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    out = np.empty(N)
    ok = np.empty(N, dtype=np.int16)
    f = None if flg is None else np.ascontiguousarray(flg, dtype=np.int16)
    lib().orc_sn_loglike(C.byref(s), N, D, X, _ptr(f), out, _ptr(ok))
    return out, ok


def lum_dist(om, ode, w0, h, z, G=8, nsub=64):
    st = C.c_int()
    d = lib().orc_lum_dist(om, ode, w0, h, z, G, nsub, C.byref(st))
    return d, st.value


def tpl_prepare(A, Cm, dobs):
    A = np.ascontiguousarray(A, dtype=np.float64)
    M, P = A.shape
    At = np.empty_like(A)
    dt = np.empty(M)
    rc = lib().orc_tpl_prepare(M, P, A, np.ascontiguousarray(Cm, dtype=np.float64),
                               np.ascontiguousarray(dobs, dtype=np.float64), At, dt)
    if rc:
        raise ValueError("template covariance not positive definite")
    return At, dt


def tpl_loglike(At, dt, X, flg=None):
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    out = np.empty(N)
    f = None if flg is None else np.ascontiguousarray(flg, dtype=np.int16)
    lib().orc_tpl_loglike(At.shape[0], D, np.ascontiguousarray(At), np.ascontiguousarray(dt), N, X, _ptr(f), out)
    return out


def logweights(beta, logpost, logq, flg):
    N = len(logq)
    out = np.empty(N)
    lib().orc_logweights(N, beta, np.ascontiguousarray(logpost, dtype=np.float64),
                         np.ascontiguousarray(logq, dtype=np.float64),
                         np.ascontiguousarray(flg, dtype=np.int16), out)
    return out


def normalize(logw, flg):
    N = len(logw)
    wbar = np.empty(N)
    ls, mw = C.c_double(), C.c_double()
    rc = lib().orc_normalize(N, np.ascontiguousarray(logw), np.ascontiguousarray(flg, dtype=np.int16),
                             wbar, C.byref(ls), C.byref(mw))
    if rc:
        raise ValueError("no sample with non-zero weight")
    return wbar, ls.value, mw.value


def perplexity(wbar, flg):
    ess = C.c_double()
    p = lib().orc_perplexity(len(wbar), np.ascontiguousarray(wbar), np.ascontiguousarray(flg, dtype=np.int16),
                             C.byref(ess))
    return p, ess.value


def enc(w):
    return lib().orc_enc(len(w), np.ascontiguousarray(w, dtype=np.float64))


def tempering_beta(kind, it, tmin, nmax):
    return lib().orc_tempering_beta(kind, it, tmin, nmax)


def update_rb(mix: Mix, X, wbar, flg, lt, logq, Q, idx, band_limit=None):
    """Returns (new Mix, dead[K]); raises on all-dead."""
    m = mix.copy()
    X = np.ascontiguousarray(X, dtype=np.float64)
    N = X.shape[0]
    dead = np.empty(m.K, dtype=np.int32)
    Qa = None if Q is None else np.ascontiguousarray(Q, dtype=np.float64)
    rc = lib().orc_update_rb(m.K, m.D, m.df, m.w, m.mu, m.L, m.logdetL, band_limit or m.D, N, X,
                             np.ascontiguousarray(wbar), np.ascontiguousarray(flg, dtype=np.int16),
                             np.ascontiguousarray(lt), np.ascontiguousarray(logq), _ptr(Qa),
                             np.ascontiguousarray(idx, dtype=np.int32), dead)
    if rc:
        raise ValueError(f"update_rb failed ({rc})")
    return m, dead


def iterate_mix(prop: Mix, target: Mix, logprior, N, seed, call, beta=1.0, bmin=None, bmax=None,
                want_sample=False, check=True):
    """One whole FP64 iteration with a Gaussian-mixture target; prop updated in place.
    check=False keeps going when the update buries every component (the work is done)."""
    st = Stats()
    X = np.empty((N, prop.D)) if want_sample else None
    logw = np.empty(N) if want_sample else None
    idx = np.empty(N, dtype=np.int32) if want_sample else None
    bmin_a = None if bmin is None else np.ascontiguousarray(bmin, dtype=np.float64)
    bmax_a = None if bmax is None else np.ascontiguousarray(bmax, dtype=np.float64)
    rc = lib().orc_iterate_mix(prop.K, prop.D, prop.df, prop.w, prop.mu, prop.L, prop.logdetL,
                               target.K, target.df, target.w, target.mu, target.L, target.logdetL,
                               float(logprior), _ptr(bmin_a), _ptr(bmax_a), N, seed, call, beta,
                               C.byref(st), _ptr(X), _ptr(logw), _ptr(idx))
    if rc and check:
        raise ValueError(f"oracle iteration failed ({rc})")
    stats = {f: getattr(st, f) for f, _ in Stats._fields_}
    return (stats, X, logw, idx) if want_sample else stats


def num_threads():
    return lib().orc_num_threads()


def prior_special(special, bmin, bmax, ind_w0=-1, ind_w1=-1, a_acc=0.0):
    """The special prior's constant (wrappers/src/param.c:1055-1101)."""
    bmin = np.ascontiguousarray(bmin, dtype=np.float64)
    bmax = np.ascontiguousarray(bmax, dtype=np.float64)
    out = C.c_double()
    rc = lib().orc_prior_special(int(special), len(bmin), bmin, bmax, int(ind_w0), int(ind_w1), float(a_acc),
                                 C.byref(out))
    if rc:
        raise ValueError("w0 range narrower than the de_conservative prior")
    return out.value


def mvdens_prior_logpdf(mean, cov, df, X, indprior=None):
    """mvdens_log_pdf of the parameters flagged by indprior (all when None), as the
    config prior of posterior_log_pdf_common (wrappers/src/param.c:1009-1026): a
    one-component mixture of weight 1 through the oracle's mixture log-pdf."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    cols = np.arange(X.shape[1]) if indprior is None else np.flatnonzero(np.asarray(indprior) == 1)
    m = Mix([1.0], np.atleast_2d(mean), cov=np.asarray(cov)[None], df=df)
    return mix_logpdf(m, np.ascontiguousarray(X[:, cols]))


def iterate_posterior(prop: Mix, logpost_fn, N, seed, call, beta=1.0, bmin=None, bmax=None, want_sample=False):
    """One whole FP64 iteration in the order of run_pmc_iteration_MPI
    (exec/cosmo_pmc.c:313-399) with any log-posterior, composed from the
    oracle's primitives (the same steps as orc_iterate_mix): the draw of
    (seed, call), log q with its per-component terms, logpost_fn(X, flg) ->
    (log posterior, ok) where ok = 0 marks a failed likelihood, the log-weights
    (non-finite ones flagged out), the normalisation, perplexity/ESS and the
    Rao-Blackwellised update. Returns (updated Mix or None when every component
    died, stats); stats["status"] is 0, or -1 when no sample had a weight and -2
    when the update buried every component. want_sample: also return the sample
    (X, unnormalised log-weights, flags, component indices)."""
    u, z, chi2 = randoms(seed, call, N, prop.D, prop.df)
    X, idx, flg, _ = draw(prop, u, z, chi2, bmin, bmax)
    logq, lt, Q = mix_logpdf(prop, X, want_terms=True)
    lp, ok = logpost_fn(X, flg)
    flg = (flg.astype(bool) & (np.asarray(ok) != 0)).astype(np.int16)
    logw = logweights(beta, lp, logq, flg)
    flg[~np.isfinite(logw)] = 0
    st = {"nok": int(flg.sum()), "status": 0}
    try:
        wbar, ls, mw = normalize(logw, flg)
    except ValueError:
        st["status"] = -1
        return None, st
    perp, ess = perplexity(wbar, flg)
    st.update(logSum=ls, maxW=mw, ln_evidence=ls - np.log(N), perplexity=perp, ess=ess)
    try:
        new, dead = update_rb(prop, X, wbar, flg, lt, logq, Q if prop.df > 0 else None, idx)
    except ValueError:
        st["status"] = -2
        return None, st
    st.update(enc=enc(new.w), ndead=int(dead.sum()))
    return (new, st, (X, logw, flg, idx)) if want_sample else (new, st)


def weighted_summary(X, wbar, flg, median=False):
    """(centre [D], limits [D, 6], status [D]) of the reference's post-processing."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    center, sigma, st = np.zeros(D), np.zeros((D, 6)), np.zeros(D, dtype=np.int32)
    lib().orc_weighted_summary(N, D, X, np.ascontiguousarray(wbar, dtype=np.float64),
                               np.ascontiguousarray(flg, dtype=np.int16), 1 if median else 0, center, sigma, st)
    return center, sigma, st


def hist1d(X, wbar, flg, nbin, lo, hi, scale):
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    h = np.zeros((D, nbin))
    lib().orc_hist1d(N, D, X, np.ascontiguousarray(wbar, dtype=np.float64), np.ascontiguousarray(flg, dtype=np.int16),
                     nbin, np.ascontiguousarray(lo, dtype=np.float64), np.ascontiguousarray(hi, dtype=np.float64),
                     scale, h)
    return h


def hist2d(X, wbar, flg, nbin, p, q, lo, hi, scale):
    X = np.ascontiguousarray(X, dtype=np.float64)
    N, D = X.shape
    h = np.zeros((nbin, nbin))
    lib().orc_hist2d(N, D, X, np.ascontiguousarray(wbar, dtype=np.float64), np.ascontiguousarray(flg, dtype=np.int16),
                     nbin, p, q, np.ascontiguousarray(lo, dtype=np.float64), np.ascontiguousarray(hi, dtype=np.float64),
                     scale, h)
    return h


def clip_weights(logw, flg, k):
    """Flags after clipping the k largest log-weights among counted samples,
    ties to the lower index (the semantics pinned for the absent pmclib
    clip_weights; exec/cosmo_pmc.c:395-399, Manual/manual.tex:636-642)."""
    logw = np.asarray(logw, dtype=np.float64)
    out = np.asarray(flg, dtype=np.int16).copy()
    cand = np.flatnonzero(out != 0)
    order = cand[np.argsort(-logw[cand], kind="stable")]
    out[order[:k]] = 0
    return out



def revive(mix: Mix, bmin, bmax, fshift, nrevive, seed, call):
    """The revive step (exec/cosmo_pmc.c:205-275) on a copy of mix; returns the new Mix."""
    m = mix.copy()
    rc = lib().orc_revive(m.K, m.D, m.w, m.mu, m.L, np.ascontiguousarray(bmin, dtype=np.float64),
                          np.ascontiguousarray(bmax, dtype=np.float64), float(fshift), int(nrevive), int(seed),
                          int(call))
    if rc:
        raise ValueError(f"revive failed ({rc})")
    return Mix(m.w, m.mu, df=m.df, L=m.L)
