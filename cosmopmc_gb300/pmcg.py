"""ctypes mirror of the libpmcg C ABI (include/pmcg.h).

The library is the product: every per-sample computation runs in its CUDA
kernels. This module only declares the structs and signatures, converts
numpy arrays, and turns the error chain into `PmcgError`. It raises when the
shared library is missing; there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpmcg.so")

FP64 = 0
MIXED = 1
SPECIAL_NONE, SPECIAL_UNITY, SPECIAL_DE_CONSERVATIVE = 0, 1, 2
DEAD_BURY, DEAD_REVIVE = 0, 1
TEMPERING_NONE, TEMPERING_LINEAR, TEMPERING_LOG = 0, 1, 2
SN_CHI2_FULL, SN_CHI2_MARG = 0, 1

ERRORS = {
    -9001: "PMCG_ECUDA", -9002: "PMCG_EDIM", -9003: "PMCG_ECHOL", -9004: "PMCG_ENOSAMPLE",
    -9005: "PMCG_ENEGWEIGHT", -9006: "PMCG_EUNSUPPORTED", -9007: "PMCG_EALLOC", -9008: "PMCG_EARG",
    -9009: "PMCG_ETIMEOUT", -9010: "PMCG_EIO", -9011: "PMCG_ENOWEIGHT", -9012: "PMCG_ESTEPS",
}


class PmcgError(RuntimeError):
    def __init__(self, code, text):
        super().__init__(f"{ERRORS.get(code, code)}: {text}")
        self.code = code


class Error(C.Structure):
    pass


Error._fields_ = [("errWhere", C.c_char * 128), ("errText", C.c_char * 384), ("errValue", C.c_int),
                  ("line", C.c_int), ("next", C.POINTER(Error))]


class Mvdens(C.Structure):
    _fields_ = [("ndim", C.c_int), ("df", C.c_int), ("mean", C.POINTER(C.c_double)),
                ("std", C.POINTER(C.c_double)), ("band_limit", C.c_int), ("chol", C.c_int), ("det", C.c_double)]


class MixMvdensS(C.Structure):
    _fields_ = [("ncomp", C.c_int), ("ndim", C.c_int), ("wght", C.POINTER(C.c_double)),
                ("comp", C.POINTER(C.POINTER(Mvdens)))]


class ParaboxS(C.Structure):
    _fields_ = [("ndim", C.c_int), ("min", C.POINTER(C.c_double)), ("max", C.POINTER(C.c_double))]


class PmcSimuS(C.Structure):
    _fields_ = [("nsamples", C.c_size_t), ("maxsamples", C.c_size_t), ("ndim", C.c_int), ("n_ded", C.c_int),
                ("X", C.POINTER(C.c_double)), ("X_ded", C.POINTER(C.c_double)),
                ("weights", C.POINTER(C.c_double)), ("flg", C.POINTER(C.c_short)),
                ("indices", C.POINTER(C.c_int)), ("isLog", C.c_int), ("logSum", C.c_double),
                ("maxW", C.c_double), ("nok", C.c_size_t), ("pinned", C.c_int)]


class RngS(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("calls", C.c_uint32)]


class SnData(C.Structure):
    _fields_ = [("nsn", C.c_int), ("z", C.c_void_p), ("mB", C.c_void_p), ("x1", C.c_void_p), ("c", C.c_void_p),
                ("cov6", C.c_void_p), ("sig_int", C.c_double), ("v_pec", C.c_double), ("h", C.c_double),
                ("chi2mode", C.c_int), ("add_logdet", C.c_int), ("quad_nodes", C.c_int),
                ("ip_Omegam", C.c_int), ("ip_Omegade", C.c_int), ("ip_w0", C.c_int), ("ip_M", C.c_int),
                ("ip_alpha", C.c_int), ("ip_beta", C.c_int),
                ("def_Omegam", C.c_double), ("def_w0", C.c_double), ("def_M", C.c_double),
                ("def_alpha", C.c_double), ("def_beta", C.c_double), ("neg_M", C.c_int), ("neg_beta", C.c_int)]


class IterStats(C.Structure):
    _fields_ = [("ln_evidence", C.c_double), ("perplexity", C.c_double), ("ess", C.c_double), ("enc", C.c_double),
                ("logSum", C.c_double), ("maxW", C.c_double), ("nok", C.c_size_t), ("ndead", C.c_int),
                ("status", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class WeightStats(C.Structure):
    _fields_ = [("logSum", C.c_double), ("maxW", C.c_double), ("ln_evidence", C.c_double),
                ("perplexity", C.c_double), ("ess", C.c_double), ("nok", C.c_size_t)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_jobs", C.c_int), ("autotune", C.c_int),
                ("dead_comp", C.c_int), ("fshift", C.c_double), ("alone_min_samples", C.c_size_t)]


class JobResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("ln_evidence", C.c_double),
                ("perplexity", C.c_double), ("ess", C.c_double), ("enc", C.c_double), ("submit_s", C.c_double),
                ("start_s", C.c_double), ("finish_s", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerInfo(C.Structure):
    _fields_ = [("queued", C.c_int), ("resident", C.c_int), ("peak_resident", C.c_int),
                ("bytes_in_use", C.c_size_t), ("peak_bytes", C.c_size_t), ("budget_bytes", C.c_size_t),
                ("epochs", C.c_longlong)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


PErr = C.POINTER(C.POINTER(Error))
_dp = C.POINTER(C.c_double)
LOGPDF_FN = C.CFUNCTYPE(C.c_double, C.c_void_p, _dp, PErr)

# (name, restype, argtypes) of every exported function
SIGNATURES = [
    ("addError", C.POINTER(Error), [C.c_int, C.c_char_p, C.POINTER(Error), C.c_int]),
    ("isError", C.c_int, [C.POINTER(Error)]),
    ("getErrorValue", C.c_int, [C.POINTER(Error)]),
    ("purgeError", None, [PErr]),
    ("printError", None, [C.c_void_p, C.POINTER(Error)]),
    ("mvdens_alloc", C.POINTER(Mvdens), [C.c_int, PErr]),
    ("mvdens_free", None, [C.POINTER(C.POINTER(Mvdens))]),
    ("mix_mvdens_alloc", C.POINTER(MixMvdensS), [C.c_int, C.c_int, PErr]),
    ("mix_mvdens_free", None, [C.POINTER(C.POINTER(MixMvdensS))]),
    ("mix_mvdens_copy", None, [C.POINTER(MixMvdensS), C.POINTER(MixMvdensS), PErr]),
    ("mvdens_cholesky_decomp", None, [C.POINTER(Mvdens), PErr]),
    ("mix_mvdens_cholesky_decomp", None, [C.POINTER(MixMvdensS), PErr]),
    ("mvdens_from_meanvar", None, [C.POINTER(Mvdens), _dp, _dp, C.c_double]),
    ("mvdens_log_pdf", C.c_double, [C.POINTER(Mvdens), _dp, PErr]),
    ("mvdens_log_pdf_void", C.c_double, [C.c_void_p, _dp, PErr]),
    ("mix_mvdens_log_pdf", C.c_double, [C.POINTER(MixMvdensS), _dp, PErr]),
    ("mix_mvdens_log_pdf_void", C.c_double, [C.c_void_p, _dp, PErr]),
    ("mix_mvdens_dump", None, [C.c_void_p, C.POINTER(MixMvdensS)]),
    ("mix_mvdens_dwnp", C.POINTER(MixMvdensS), [C.c_void_p, PErr]),
    ("mix_mvdens_print", None, [C.c_void_p, C.POINTER(MixMvdensS)]),
    ("out_pmc_simu_cosmo_pmc", None, [C.c_char_p, C.POINTER(PmcSimuS), C.c_void_p, C.c_double, PErr]),
    ("pmcg_set_par_names", None, [C.c_int, C.POINTER(C.c_char_p)]),
    ("pmcg_out_pmc_simu_names", None, [C.c_char_p, C.POINTER(PmcSimuS), C.POINTER(C.c_char_p), PErr]),
    ("pmcg_set_rng_seed_hook", None, [C.c_void_p]),
    ("pmcg_rng_forget", None, [C.c_void_p]),
    ("pmcg_register_posterior", None, [C.c_void_p, C.c_void_p]),
    ("pmcg_posterior_from_config", C.c_void_p, [C.c_int, C.POINTER(C.c_int), _dp, _dp, C.c_int, C.POINTER(C.c_int),
                                                C.POINTER(C.c_void_p), C.POINTER(Mvdens), C.POINTER(C.c_int),
                                                C.c_double, PErr]),
    ("pmc_simu_from_file", C.POINTER(PmcSimuS), [C.c_void_p, C.c_size_t, C.c_int, C.c_int,
                                                   C.POINTER(MixMvdensS), C.c_int, PErr]),
    ("importance_sample", C.c_size_t, [C.POINTER(PmcSimuS), C.c_void_p, C.c_int, PErr]),
    ("pmcg_weighted_moments", None, [C.POINTER(PmcSimuS), _dp, _dp, PErr]),
    ("pmcg_weighted_summary", None, [C.POINTER(PmcSimuS), C.c_int, _dp, _dp, PErr]),
    ("pmcg_weighted_hist1d", None, [C.POINTER(PmcSimuS), C.c_int, _dp, _dp, _dp, PErr]),
    ("pmcg_weighted_hist2d", None, [C.POINTER(PmcSimuS), C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, PErr]),
    ("effective_number_of_components", C.c_double, [C.POINTER(MixMvdensS), PErr]),
    ("init_parabox", C.POINTER(ParaboxS), [C.c_int, PErr]),
    ("add_slab", None, [C.POINTER(ParaboxS), C.c_int, C.c_double, C.c_double, PErr]),
    ("free_parabox", None, [C.POINTER(C.POINTER(ParaboxS))]),
    ("isinBox", C.c_int, [C.POINTER(ParaboxS), _dp]),
    ("pmc_simu_init_mpi", C.POINTER(PmcSimuS), [C.c_size_t, C.c_int, C.c_int, PErr]),
    ("pmc_simu_init_plus_ded", C.POINTER(PmcSimuS), [C.c_size_t, C.c_int, C.c_int, PErr]),
    ("pmc_simu_realloc", None, [C.POINTER(PmcSimuS), C.c_size_t, PErr]),
    ("pmc_simu_free", None, [C.POINTER(C.POINTER(PmcSimuS))]),
    ("pmcg_rng_alloc", C.POINTER(RngS), [C.c_uint64]),
    ("pmcg_rng_free", None, [C.POINTER(C.POINTER(RngS))]),
    ("simulate_mix_mvdens", C.c_size_t, [C.POINTER(PmcSimuS), C.POINTER(MixMvdensS), C.c_void_p,
                                         C.POINTER(ParaboxS), PErr]),
    ("generic_get_importance_weight_and_deduced_verb", C.c_size_t,
     [C.POINTER(PmcSimuS), C.POINTER(MixMvdensS), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
      C.c_int, PErr]),
    ("normalize_importance_weight", C.c_double, [C.POINTER(PmcSimuS), PErr]),
    ("update_prop_rb", None, [C.POINTER(MixMvdensS), C.POINTER(PmcSimuS), PErr]),
    ("perplexity_and_ess", C.c_double, [C.POINTER(PmcSimuS), C.c_int, _dp, PErr]),
    ("evidence", C.c_double, [C.POINTER(PmcSimuS), _dp, PErr]),
    ("get_tempering_beta", C.c_double, [C.c_int, C.c_int, C.c_double, C.c_int, PErr]),
    ("pmcg_simu_host_modified", None, [C.POINTER(PmcSimuS)]),
    ("pmcg_simu_set_precision", None, [C.POINTER(PmcSimuS), C.c_int, PErr]),
    ("pmcg_simu_set_tensor_cores", None, [C.POINTER(PmcSimuS), C.c_int, PErr]),
    ("pmcg_set_dropin_precision", None, [C.c_int]),
    ("pmcg_set_tensor_cores", C.c_int, [C.c_int]),
    ("pmcg_posterior_alloc", C.c_void_p, [C.c_int, _dp, _dp, PErr]),
    ("pmcg_posterior_free", None, [C.POINTER(C.c_void_p)]),
    ("pmcg_posterior_add_mixmvdens", None, [C.c_void_p, C.POINTER(MixMvdensS), PErr]),
    ("pmcg_posterior_add_snia", None, [C.c_void_p, C.POINTER(SnData), PErr]),
    ("pmcg_posterior_add_template", None, [C.c_void_p, C.c_int, _dp, _dp, _dp, PErr]),
    ("pmcg_posterior_set_special", None, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, PErr]),
    ("pmcg_posterior_add_mvdens_prior", None, [C.c_void_p, C.POINTER(Mvdens), C.POINTER(C.c_int), PErr]),
    ("pmcg_posterior_log_pdf_void", C.c_double, [C.c_void_p, _dp, PErr]),
    ("pmcg_fisher_matrix", C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int, _dp, PErr]),
    ("clip_weights", None, [C.POINTER(PmcSimuS), C.c_int, C.c_void_p, PErr]),
    ("pmcg_max_posterior", C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_double, C.c_int, _dp, _dp, PErr]),
    ("pmcg_fisher_proposal", None, [C.POINTER(MixMvdensS), _dp, _dp, _dp, _dp, C.c_int, C.c_double, C.c_double,
                                    C.POINTER(RngS), PErr]),
    ("pmcg_posterior_log_pdf_batch", None, [C.c_void_p, C.c_size_t, _dp, _dp, C.POINTER(C.c_short), C.c_int,
                                            C.c_int, C.c_void_p, PErr]),
    ("pmcg_mix_log_pdf_batch", None, [C.POINTER(MixMvdensS), C.c_size_t, _dp, _dp, _dp, C.c_int, PErr]),
    ("pmcg_run_create", C.c_void_p, [C.POINTER(MixMvdensS), C.c_void_p, C.POINTER(ParaboxS), C.c_size_t, C.c_int,
                                     C.c_uint64, PErr]),
    ("pmcg_run_iterate", None, [C.c_void_p, C.c_double, C.POINTER(IterStats), PErr]),
    ("pmcg_run_iterate_async", None, [C.c_void_p, C.c_double, PErr]),
    ("pmcg_run_iterate_wait", None, [C.c_void_p, C.POINTER(IterStats), PErr]),
    ("pmcg_run_get_proposal", None, [C.c_void_p, C.POINTER(MixMvdensS), PErr]),
    ("pmcg_run_get_sample", None, [C.c_void_p, C.POINTER(PmcSimuS), PErr]),
    ("pmcg_run_set_dead_comp", None, [C.c_void_p, C.c_int, C.c_double, PErr]),
    ("pmcg_run_set_tensor_cores", C.c_int, [C.c_void_p, C.c_int, PErr]),
    ("pmcg_run_set_proposal", None, [C.c_void_p, C.POINTER(MixMvdensS), PErr]),
    ("pmcg_run_free", None, [C.POINTER(C.c_void_p)]),
    ("pmcg_run_set_timing", None, [C.c_void_p, C.c_int]),
    ("pmcg_run_stage_ms", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("pmcg_run_iteration_ms", C.c_int, [C.c_void_p, _dp]),
    ("pmcg_run_last_launches", C.c_int, [C.c_void_p]),
    ("pmcg_run_time_stage", C.c_double, [C.c_void_p, C.c_int, C.c_int, PErr]),
    ("pmcg_batch_create", C.c_void_p, [C.c_int, C.POINTER(C.c_void_p), PErr]),
    ("pmcg_batch_rebind", None, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), PErr]),
    ("pmcg_batch_iterate", None, [C.c_void_p, _dp, C.POINTER(IterStats), PErr]),
    ("pmcg_batch_autotune", None, [C.c_void_p, PErr]),
    ("pmcg_batch_config", None, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_int)]),
    ("pmcg_batch_sn_block", C.c_int, [C.c_void_p]),
    ("pmcg_batch_last_ms", C.c_double, [C.c_void_p]),
    ("pmcg_batch_set_stage_timing", None, [C.c_void_p, C.c_int]),
    ("pmcg_batch_stage_ms", C.c_int, [C.c_void_p, _dp]),
    ("pmcg_batch_free", None, [C.POINTER(C.c_void_p)]),
    ("pmcg_server_create", C.c_void_p, [C.POINTER(ServerOpts), PErr]),
    ("pmcg_server_submit", C.c_int64, [C.c_void_p, C.POINTER(MixMvdensS), C.c_void_p, C.POINTER(ParaboxS),
                                       C.c_size_t, C.c_int, C.c_int, C.c_double, C.c_uint64, PErr]),
    ("pmcg_server_wait", C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(JobResult),
                                   C.POINTER(MixMvdensS), PErr]),
    ("pmcg_server_info", None, [C.c_void_p, C.POINTER(ServerInfo)]),
    ("pmcg_server_free", None, [C.POINTER(C.c_void_p)]),
    ("pmcg_importance_weights_noalloc", None, [C.c_size_t, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.POINTER(WeightStats), C.c_void_p, PErr]),
    ("pmcg_version", C.c_char_p, []),
    ("pmcg_device_count", C.c_int, []),
    ("pmcg_device_synchronize", None, [PErr]),
]

_lib = None


def load(path: str | None = None):
    """Load libpmcg.so (built in-tree); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libpmcg.so not built at {p}: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class _Err:
    """Holds an `error*` for one call and raises on a non-empty chain."""

    def __init__(self):
        self.p = C.POINTER(Error)()

    @property
    def ref(self):
        return C.byref(self.p)

    def check(self):
        if self.p:
            code, text = self.p.contents.errValue, self.p.contents.errText.decode(errors="replace")
            load().purgeError(C.byref(self.p))
            raise PmcgError(code, text)


def call(name, *args):
    e = _Err()
    r = getattr(load(), name)(*args, e.ref)
    e.check()
    return r


_LIBC = None


def _libc():
    global _LIBC
    if _LIBC is None:
        _LIBC = C.CDLL(None)
        _LIBC.fopen.restype = C.c_void_p
        _LIBC.fopen.argtypes = [C.c_char_p, C.c_char_p]
        _LIBC.fclose.argtypes = [C.c_void_p]
    return _LIBC


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ----------------------------------------------------------------- mixtures
class MixMvdens:
    """Owning wrapper of a `mix_mvdens*` (covariances or Cholesky factors)."""

    def __init__(self, ncomp, ndim):
        self.p = call("mix_mvdens_alloc", ncomp, ndim)
        self.K, self.D = ncomp, ndim

    @classmethod
    def from_arrays(cls, w, mu, cov=None, df=-1, L=None):
        mu = _f64(mu)
        K, D = mu.shape
        m = cls(K, D)
        m.set(w, mu, cov=cov, df=df, L=L)
        return m

    def set(self, w, mu, cov=None, df=-1, L=None):
        s = self.p.contents
        w = _f64(w)
        for k in range(self.K):
            s.wght[k] = float(w[k])
            c = s.comp[k].contents
            c.df = int(df)
            c.band_limit = self.D
            for i in range(self.D):
                c.mean[i] = float(mu[k, i])
            M = _f64(L[k] if L is not None else cov[k]).ravel()
            C.memmove(c.std, M.ctypes.data, 8 * self.D * self.D)
            c.chol = 1 if L is not None else 0
            if L is not None:
                c.det = 2.0 * float(np.sum(np.log(np.diag(L[k]))))
        return self

    def cholesky(self):
        call("mix_mvdens_cholesky_decomp", self.p)
        return self

    def arrays(self):
        """(w[K], mu[K,D], L[K,D,D] lower Cholesky) as numpy copies."""
        s = self.p.contents
        K, D = self.K, self.D
        w = np.array([s.wght[k] for k in range(K)])
        mu = np.empty((K, D))
        L = np.empty((K, D, D))
        for k in range(K):
            c = s.comp[k].contents
            mu[k] = np.ctypeslib.as_array(c.mean, shape=(D,))
            A = np.ctypeslib.as_array(c.std, shape=(D, D)).copy()
            L[k] = np.tril(A) if c.chol else np.linalg.cholesky(A)
        return w, mu, L

    @property
    def df(self):
        return self.p.contents.comp[0].contents.df

    def free(self):
        if self.p:
            load().mix_mvdens_free(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Parabox:
    def __init__(self, bmin, bmax):
        bmin, bmax = _f64(bmin), _f64(bmax)
        self.p = call("init_parabox", len(bmin))
        for i in range(len(bmin)):
            call("add_slab", self.p, i, float(bmin[i]), float(bmax[i]))
        self.min, self.max = bmin, bmax

    def free(self):
        if self.p:
            load().free_parabox(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PmcSimu:
    """Owning wrapper of a `pmc_simu*` with numpy views of its arrays."""

    def __init__(self, nsamples, ndim, n_ded=0):
        self.p = call("pmc_simu_init_mpi", nsamples, ndim, n_ded)

    @property
    def s(self):
        return self.p.contents

    @property
    def N(self):
        return self.s.nsamples

    @property
    def X(self):
        return np.ctypeslib.as_array(self.s.X, shape=(self.N, self.s.ndim))

    @property
    def weights(self):
        return np.ctypeslib.as_array(self.s.weights, shape=(self.N,))

    @property
    def flg(self):
        return np.ctypeslib.as_array(self.s.flg, shape=(self.N,))

    @property
    def indices(self):
        return np.ctypeslib.as_array(self.s.indices, shape=(self.N,))

    def host_modified(self):
        load().pmcg_simu_host_modified(self.p)

    def set_precision(self, prec):
        """Precision of the drop-in calls on this sample (FP64, MIXED, or -1:
        the process default of set_dropin_precision)."""
        call("pmcg_simu_set_precision", self.p, int(prec))

    def set_tensor_cores(self, on):
        """Tensor cores for the drop-in calls on this sample (True / False, or
        None: the process default)."""
        call("pmcg_simu_set_tensor_cores", self.p, -1 if on is None else (1 if on else 0))

    def write(self, path, par_names=None):
        """CosmoPMC sample file (out_pmc_simu_cosmo_pmc)."""
        names = None
        if par_names is not None:
            names = (C.c_char_p * len(par_names))(*[n.encode() for n in par_names])
        call("pmcg_out_pmc_simu_names", str(path).encode(), self.p, names)

    @classmethod
    def read(cls, path, nsamples, ndim, n_ded=0, nclipw=0):
        """pmc_simu_from_file: normalised weights (isLog = 0), logSum, indices;
        nclipw > 0: the nclipw largest weights clipped (clip_weights)."""
        f = _libc().fopen(str(path).encode(), b"r")
        if not f:
            raise OSError(f"cannot open {path}")
        try:
            p = call("pmc_simu_from_file", f, nsamples, ndim, n_ded, None, int(nclipw))
        finally:
            _libc().fclose(f)
        obj = cls.__new__(cls)
        obj.p = p
        return obj

    def importance_sample(self, post, quiet=1):
        """Weights := log-posterior of each sample (importance_sample)."""
        return call("importance_sample", self.p, post.p, quiet)

    def weighted_moments(self):
        D = self.s.ndim
        mean, cov = np.empty(D), np.empty((D, D))
        call("pmcg_weighted_moments", self.p, _dptr(mean), _dptr(cov))
        return mean, cov

    def weighted_summary(self, median=False):
        """(centre [D], limits [D, 6]): weighted mean (or median) of every parameter and
        the one-sided 68.27/95.45/99.73 % limits right then left of it (-1: sample ended)."""
        D = self.s.ndim
        center, sigma = np.empty(D), np.empty((D, 6))
        call("pmcg_weighted_summary", self.p, 1 if median else 0, _dptr(center), _dptr(sigma))
        return center, sigma

    def weighted_hist1d(self, nbin, lo, hi):
        """[D, nbin] weighted histograms (normalised weights x nsamples) over [lo, hi]."""
        D = self.s.ndim
        lo, hi = _f64(lo), _f64(hi)
        h = np.empty((D, nbin))
        call("pmcg_weighted_hist1d", self.p, nbin, _dptr(lo), _dptr(hi), _dptr(h))
        return h

    def weighted_hist2d(self, nbin, p, q, lo, hi):
        """[nbin, nbin] weighted histogram of parameters (p, q) over [lo, hi]."""
        lo, hi = _f64(lo), _f64(hi)
        h = np.empty((nbin, nbin))
        call("pmcg_weighted_hist2d", self.p, nbin, p, q, _dptr(lo), _dptr(hi), _dptr(h))
        return h

    def free(self):
        if self.p:
            load().pmc_simu_free(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Rng:
    def __init__(self, seed):
        self.p = load().pmcg_rng_alloc(seed)

    @property
    def calls(self):
        return self.p.contents.calls

    def __del__(self):
        try:
            load().pmcg_rng_free(C.byref(self.p))
        except Exception:
            pass


# ----------------------------------------------------------------- posterior
class Posterior:
    def __init__(self, npar, bmin=None, bmax=None):
        self._keep = []
        if bmin is not None:
            bmin, bmax = _f64(bmin), _f64(bmax)
            self.p = C.c_void_p(call("pmcg_posterior_alloc", npar, _dptr(bmin), _dptr(bmax)))
        else:
            self.p = C.c_void_p(call("pmcg_posterior_alloc", npar, None, None))
        self.npar = npar

    def add_mix(self, target: MixMvdens):
        call("pmcg_posterior_add_mixmvdens", self.p, target.p)
        return self

    def fisher(self, pos, bmin, bmax, diag_only=False, force_positive=False, with_positive=False):
        """Fisher matrix -d^2 log P at pos (central differences, steps 0.001 (bmax - bmin)).
        with_positive: also return whether F is positive definite."""
        pos, bmin, bmax = _f64(pos), _f64(bmin), _f64(bmax)
        F = np.empty((self.npar, self.npar))
        pd = call("pmcg_fisher_matrix", self.p, _dptr(pos), _dptr(bmin), _dptr(bmax), int(diag_only),
                  int(force_positive), _dptr(F))
        return (F, bool(pd == 1)) if with_positive else F

    def max_posterior(self, starts, bmin, bmax, ftol=1e-8, max_evals=5000):
        """Nelder-Mead searches for the maximum of log P from each row of starts
        (advanced together, trial points evaluated in batches on the device).
        Returns (best point, its log P, every search's best points, their log P)."""
        starts = np.ascontiguousarray(np.atleast_2d(starts), dtype=np.float64)
        bmin, bmax = _f64(bmin), _f64(bmax)
        ns = starts.shape[0]
        best = np.empty((ns, self.npar))
        lp = np.empty(ns)
        i = call("pmcg_max_posterior", self.p, ns, _dptr(starts), _dptr(bmin), _dptr(bmax), float(ftol),
                 int(max_evals), _dptr(best), _dptr(lp))
        return best[i].copy(), float(lp[i]), best, lp

    def add_snia(self, sn: dict):
        s = SnData()
        arrs = {k: _f64(sn[k]) for k in ("z", "mB", "x1", "c", "cov6")}
        self._keep.append(arrs)
        s.nsn = len(arrs["z"])
        for k, a in arrs.items():
            setattr(s, k, a.ctypes.data)
        for k in ("sig_int", "v_pec", "h"):
            setattr(s, k, float(sn[k]))
        s.chi2mode, s.add_logdet, s.quad_nodes = int(sn["chi2mode"]), int(sn["add_logdet"]), int(sn["quad_nodes"])
        s.ip_Omegam, s.ip_Omegade, s.ip_w0 = int(sn["ip_om"]), int(sn["ip_ode"]), int(sn["ip_w0"])
        s.ip_M, s.ip_alpha, s.ip_beta = int(sn["ip_M"]), int(sn["ip_alpha"]), int(sn["ip_beta"])
        s.def_Omegam, s.def_w0, s.def_M = float(sn["def_om"]), float(sn["def_w0"]), float(sn["def_M"])
        s.def_alpha, s.def_beta = float(sn["def_alpha"]), float(sn["def_beta"])
        s.neg_M, s.neg_beta = int(sn.get("neg_M", 0)), int(sn.get("neg_beta", 0))
        call("pmcg_posterior_add_snia", self.p, C.byref(s))
        return self

    def set_special(self, special, ind_w0=-1, ind_w1=-1, a_acc=0.0):
        """Special prior (SPECIAL_NONE / SPECIAL_UNITY / SPECIAL_DE_CONSERVATIVE)."""
        call("pmcg_posterior_set_special", self.p, int(special), int(ind_w0), int(ind_w1), float(a_acc))
        return self

    def add_prior(self, mean, cov, df=-1, indprior=None):
        """Gaussian (df <= 0) or Student-t prior on the parameters flagged by indprior."""
        mean, cov = _f64(mean), _f64(cov)
        d = len(mean)
        m = Mvdens()
        m.ndim, m.df, m.band_limit, m.chol, m.det = d, int(df), d, 0, 0.0
        m.mean = _dptr(mean)
        m.std = _dptr(cov)
        ind = None
        if indprior is not None:
            ind = np.ascontiguousarray(indprior, dtype=np.int32)
        call("pmcg_posterior_add_mvdens_prior", self.p, C.byref(m),
             None if ind is None else ind.ctypes.data_as(C.POINTER(C.c_int)))
        return self

    def add_template(self, A, Cm, dobs):
        A, Cm, dobs = _f64(A), _f64(Cm), _f64(dobs)
        call("pmcg_posterior_add_template", self.p, A.shape[0], _dptr(A), _dptr(Cm), _dptr(dobs))
        return self

    def log_pdf_batch(self, X, precision=FP64):
        X = _f64(X)
        N = X.shape[0]
        out = np.empty(N)
        flg = np.empty(N, dtype=np.int16)
        call("pmcg_posterior_log_pdf_batch", self.p, N, _dptr(X), _dptr(out),
             flg.ctypes.data_as(C.POINTER(C.c_short)), 0, precision, None)
        return out, flg

    def free(self):
        if self.p:
            load().pmcg_posterior_free(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def mix_log_pdf_batch(mix: MixMvdens, X, precision=FP64, want_terms=False):
    X = _f64(X)
    N = X.shape[0]
    logq = np.empty(N)
    lt = np.empty((mix.K, N)) if want_terms else None
    call("pmcg_mix_log_pdf_batch", mix.p, N, _dptr(X), _dptr(logq), None if lt is None else _dptr(lt), precision)
    return (logq, lt) if want_terms else logq


# ----------------------------------------------------------------- runs
class Run:
    """Device-resident PMC run (pmcg_run_*)."""

    def __init__(self, proposal: MixMvdens, posterior: Posterior, nsamples, precision=FP64, seed=1, box=None):
        self.p = C.c_void_p(call("pmcg_run_create", proposal.p, posterior.p, box.p if box is not None else None,
                                 nsamples, precision, seed))
        self.K, self.D, self.N = proposal.K, proposal.D, nsamples
        self.df = proposal.df
        self._post = posterior

    def iterate(self, beta=1.0):
        st = IterStats()
        call("pmcg_run_iterate", self.p, beta, C.byref(st))
        return st.as_dict()

    def iterate_async(self, beta=1.0):
        """Start an iteration (pmcg_run_iterate_async); finish it with iterate_wait."""
        call("pmcg_run_iterate_async", self.p, beta)

    def iterate_wait(self):
        st = IterStats()
        call("pmcg_run_iterate_wait", self.p, C.byref(st))
        return st.as_dict()

    def proposal(self) -> MixMvdens:
        m = MixMvdens(self.K, self.D)
        call("pmcg_run_get_proposal", self.p, m.p)
        return m

    def set_dead_comp(self, mode, fshift=0.1):
        """DEAD_BURY (default) or DEAD_REVIVE (revive_comp, needs the run's box)."""
        call("pmcg_run_set_dead_comp", self.p, int(mode), float(fshift))

    def set_tensor_cores(self, on):
        """This run's tensor-core setting (True / False, or None: the process
        default of set_tensor_cores); returns the previous one (None, 0 or 1)."""
        prev = call("pmcg_run_set_tensor_cores", self.p, -1 if on is None else (1 if on else 0))
        return None if prev < 0 else prev

    def set_proposal(self, m: MixMvdens):
        call("pmcg_run_set_proposal", self.p, m.p)

    def sample(self) -> PmcSimu:
        ps = PmcSimu(self.N, self.D)
        call("pmcg_run_get_sample", self.p, ps.p)
        return ps

    def set_timing(self, on=True, stages=True):
        """CUDA-event timing: per stage (every kernel launched directly) or, with
        stages=False, whole iterations as they run in production (one replayed
        CUDA graph per single-precision iteration)."""
        load().pmcg_run_set_timing(self.p, (1 if stages else 2) if on else 0)

    def stage_ms(self):
        ms = (C.c_double * 5)()
        n = load().pmcg_run_stage_ms(self.p, ms, 5)
        return list(ms), n

    def iteration_ms(self):
        """(summed ms of the timed iterations, their number)."""
        ms = C.c_double()
        n = load().pmcg_run_iteration_ms(self.p, C.byref(ms))
        return ms.value, n

    def last_launches(self):
        return load().pmcg_run_last_launches(self.p)

    def time_stage(self, stage, reps=10):
        """Mean ms of re-evaluating stage 1 (log q) or 2 (log posterior) of the current sample."""
        return call("pmcg_run_time_stage", self.p, stage, reps)

    def free(self):
        if self.p:
            load().pmcg_run_free(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """Many runs iterated by one persistent launch (pmcg_batch_*); holds the runs alive."""

    def __init__(self, runs):
        self.runs = list(runs)
        arr = (C.c_void_p * len(self.runs))(*[r.p.value for r in self.runs])
        self.p = C.c_void_p(call("pmcg_batch_create", len(self.runs), arr))

    def rebind(self, runs):
        """Iterate another set of runs with this batch (pmcg_batch_rebind)."""
        runs = list(runs)
        arr = (C.c_void_p * len(runs))(*[r.p.value for r in runs])
        call("pmcg_batch_rebind", self.p, len(runs), arr)
        self.runs = runs

    def iterate(self, betas=None):
        R = len(self.runs)
        st = (IterStats * R)()
        b = None if betas is None else _dptr(_f64(betas))
        call("pmcg_batch_iterate", self.p, b, st)
        return [s.as_dict() for s in st]

    def autotune(self):
        call("pmcg_batch_autotune", self.p)

    def config(self):
        v = [C.c_int() for _ in range(4)]
        load().pmcg_batch_config(self.p, *[C.byref(x) for x in v])
        return dict(samples_per_thread=v[0].value, blocks_per_sm=v[1].value, grid=v[2].value, graph=v[3].value,
                    sn_threads=load().pmcg_batch_sn_block(self.p))

    def last_ms(self):
        return load().pmcg_batch_last_ms(self.p)

    BATCH_STAGES = ("draw", "logq", "logpost", "prior", "weight_tiles", "weight_merge", "em_factor", "em_stats",
                    "em_finalise", "prep_comp", "renorm", "prep_consts")

    def set_stage_timing(self, on):
        load().pmcg_batch_set_stage_timing(self.p, 1 if on else 0)

    def stage_ms(self):
        """Per-stage ms of the last iteration (stage timing on), else None."""
        ms = np.zeros(len(self.BATCH_STAGES))
        if load().pmcg_batch_stage_ms(self.p, _dptr(ms)) != 0:
            return None
        return dict(zip(self.BATCH_STAGES, ms.tolist()))

    def free(self):
        if self.p:
            load().pmcg_batch_free(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Continuous-batching PMC server (pmcg_server_*)."""

    def __init__(self, hbm_budget_bytes=0, max_jobs=0, autotune=False, dead_comp=DEAD_BURY, fshift=0.1,
                 alone_min_samples=0):
        o = ServerOpts(hbm_budget_bytes, max_jobs, 1 if autotune else 0, dead_comp, fshift, alone_min_samples)
        self.p = C.c_void_p(call("pmcg_server_create", C.byref(o)))
        self._keep = {}

    def submit(self, proposal: MixMvdens, posterior: Posterior, nsamples, niter, seed, box=None,
               tempering=TEMPERING_NONE, t_min=0.0):
        jid = call("pmcg_server_submit", self.p, proposal.p, posterior.p, box.p if box is not None else None,
                   nsamples, niter, tempering, t_min, seed)
        self._keep[jid] = (proposal.K, proposal.D, posterior)
        return jid

    def wait(self, jid, timeout=60.0, want_proposal=False):
        res = JobResult()
        K, D, _ = self._keep[jid]
        m = MixMvdens(K, D) if want_proposal else None
        r = call("pmcg_server_wait", self.p, jid, timeout, C.byref(res), m.p if m is not None else None)
        out = res.as_dict()
        out["finished"] = r == 1
        return (out, m) if want_proposal else out

    def info(self):
        i = ServerInfo()
        load().pmcg_server_info(self.p, C.byref(i))
        return i.as_dict()

    def free(self):
        if self.p:
            load().pmcg_server_free(C.byref(self.p))
            self.p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ----------------------------------------------------------------- drop-in calls
def simulate_mix_mvdens(psim: PmcSimu, prop: MixMvdens, rng: Rng, pb: Parabox | None = None):
    return call("simulate_mix_mvdens", psim.p, prop.p, rng.p, pb.p if pb is not None else None)


def importance_weights(psim: PmcSimu, prop: MixMvdens, post: Posterior, beta=1.0):
    L = load()
    q = C.cast(L.mix_mvdens_log_pdf_void, C.c_void_p)
    f = C.cast(L.pmcg_posterior_log_pdf_void, C.c_void_p)
    return call("generic_get_importance_weight_and_deduced_verb", psim.p, prop.p, q, f, None, post.p, beta, 1)


def normalize_importance_weight(psim: PmcSimu):
    return call("normalize_importance_weight", psim.p)


def clip_weights(psim: PmcSimu, nclipw: int):
    """Flag out the nclipw largest weights (ties to the lower index); a
    normalised sample is renormalised over the samples kept."""
    call("clip_weights", psim.p, int(nclipw), None)


def update_prop_rb(prop: MixMvdens, psim: PmcSimu):
    call("update_prop_rb", prop.p, psim.p)


def perplexity_and_ess(psim: PmcSimu):
    ess = C.c_double()
    p = call("perplexity_and_ess", psim.p, 1, C.byref(ess))
    return p, ess.value


def evidence(psim: PmcSimu):
    ln = C.c_double()
    e = call("evidence", psim.p, C.byref(ln))
    return e, ln.value


def effective_number_of_components(prop: MixMvdens):
    return call("effective_number_of_components", prop.p)


def get_tempering_beta(kind, it, tmin, nmax):
    return call("get_tempering_beta", kind, it, tmin, nmax)


def set_dropin_precision(prec):
    load().pmcg_set_dropin_precision(prec)


def set_tensor_cores(on):
    """Switch the single-precision mixture log-density (D <= 32) between the
    tcgen05 tensor-core kernel and the CUDA-core kernel; returns the previous
    setting."""
    return load().pmcg_set_tensor_cores(1 if on else 0)


def device_count():
    return load().pmcg_device_count()


FISHER_RSHIFT, FISHER_EIGEN = 0, 1


def fisher_proposal(prop: MixMvdens, F, pos, bmin, bmax, kind=FISHER_EIGEN, fshift=0.1, fvar=1.0, rng=None):
    """Fill prop (means, covariances fvar F^-1, equal weights) from a Fisher matrix."""
    F, pos, bmin, bmax = _f64(F), _f64(pos), _f64(bmin), _f64(bmax)
    call("pmcg_fisher_proposal", prop.p, _dptr(F), _dptr(pos), _dptr(bmin), _dptr(bmax), kind, fshift, fvar,
         rng.p if rng is not None else None)
    return prop
