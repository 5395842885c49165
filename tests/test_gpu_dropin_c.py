"""The drop-in boundary from C: tests/c/dropin_sequence.c, compiled with gcc
against include/pmcg.h and linked to libpmcg.so, runs the CosmoPMC driver's
one-process iteration sequence (run_pmc_iteration_MPI, exec/cosmo_pmc.c:
293-402, with post_processing's diagnostics) on an SN Ia configuration in the
reference's own conventions: parameters Omega_m, w_0_de, -M, alpha, -beta (the
-M and -beta storage of par_files/cosmo_SN.par:9; the parameter set of
Demo/MC_Demo/SN/config_pmc), SN_SALT stretch s = x1 + 1, a flat universe (no
Omega_de parameter), the caller's own generator through the seed hook, its own
posterior callback with &config registered for the device posterior built by
pmcg_posterior_from_config, and the sample file written with its par_t codes.

Every iteration is compared with the FP64 oracle (same draw: the generator's
stream key is the caller's seed, the call count the iteration), continuing
from the C program's updated proposal: counts exactly, ln Z to 1e-8 relative,
perplexity/ESS/ENC to 1e-6, proposals to 1e-7 of the component's standard
deviations, and the
sample file row by row (unnormalised log-weight, -component, parameters)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cosmopmc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PAR = [0, 14, 37, 38, 39]                 # p_Omegam, p_w0de, p_M, p_alpha, p_beta
BMIN = np.array([0.0, -3.0, 18.5, 0.0, -5.0])
BMAX = np.array([1.2, 0.0, 20.0, 0.4, -1.0])
TRUTH = np.array([0.3, -1.0, 19.1, 0.14, -3.1])   # (Omega_m, w0, -M, alpha, -beta)


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    gcc = shutil.which("gcc")
    assert gcc, "gcc is needed to build the C caller"
    lib_dir = os.path.join(ROOT, "cosmopmc_gb300")
    out = tmp_path_factory.mktemp("cbin") / "dropin_sequence"
    r = subprocess.run([gcc, "-std=c11", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "c", "dropin_sequence.c"), "-L", lib_dir, "-lpmcg",
                        f"-Wl,-rpath,{lib_dir}", "-lm", "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


def _inputs(K=5, N=20000, niter=3, seed=5150, beta=1.0):
    sn = W.sn_data()
    s = sn["x1"] + 1.0   # stretch form
    rng = np.random.default_rng(7)
    sd = np.array([0.05, 0.2, 0.04, 0.02, 0.15])
    mu = TRUTH[None, :] + 0.5 * sd[None, :] * rng.standard_normal((K, 5))
    cov = np.repeat(np.diag((2 * sd) ** 2)[None], K, axis=0)
    lines = [f"5 {niter} {N} {seed} {float(beta)!r}", " ".join(map(str, PAR)),
             " ".join(repr(float(v)) for v in BMIN), " ".join(repr(float(v)) for v in BMAX), str(len(sn["z"]))]
    for i in range(len(sn["z"])):
        lines.append(" ".join(repr(float(v)) for v in
                              [sn["z"][i], sn["mB"][i], s[i], sn["c"][i], *sn["cov6"][i]]))
    # Theta2 defaults (-M, alpha, -beta), sig_int, v_pec, h, Omega_m, w0, chi2mode, add_logdet, nodes, special
    lines.append("19.3 0.13 -3.0 0.0 0.0 0.7 0.3 -1.0 0 0 4 0")
    lines.append(f"{K} -1")
    for k in range(K):
        lines.append(" ".join(repr(float(v)) for v in [1.0 / K, *mu[k], *cov[k].ravel()]))
    return sn, s, mu, cov, "\n".join(lines), dict(K=K, N=N, niter=niter, seed=seed, beta=beta)


def _parse(stdout, K, D):
    iters, comps = {}, {}
    for ln in stdout.splitlines():
        t = ln.split()
        if t[0] == "iter":
            iters[int(t[1])] = dict(nok=int(t[2]), ln_evidence=float(t[3]), perplexity=float(t[4]),
                                    ess=float(t[5]), enc=float(t[6]), logSum=float(t[7]))
        elif t[0] == "comp":
            it, k, chol = int(t[1]), int(t[2]), int(t[3])
            v = np.array([float(x) for x in t[4:]])
            comps.setdefault(it, [None] * K)[k] = (chol, v[0], v[1:1 + D], v[1 + D:].reshape(D, D))
    return iters, comps


def test_c_caller_runs_the_driver_sequence_like_the_oracle(binary, oracle, tmp_path):
    sn, s, mu, cov, text, cfg = _inputs()
    K, N, D = cfg["K"], cfg["N"], 5
    r = subprocess.run([binary], input=text + f"\n{tmp_path}\n", capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    iters, comps = _parse(r.stdout, K, D)
    assert sorted(iters) == list(range(cfg["niter"]))
    # the oracle in the reference's conventions: -M and -beta stored, x1 = s - 1, flat
    osn = dict(sn)
    osn.update(x1=s - 1.0, ip_om=0, ip_ode=-1, ip_w0=1, ip_M=2, ip_alpha=3, ip_beta=4, neg_M=1, neg_beta=1,
               def_om=0.3, def_w0=-1.0, def_M=-19.3, def_alpha=0.13, def_beta=3.0, quad_nodes=4, chi2mode=0)
    logpr = -np.sum(np.log(BMAX - BMIN))

    def lpf(X, flg):
        l, ok = oracle.sn_loglike(osn, X, flg)
        return l + logpr, ok

    om = oracle.Mix(np.full(K, 1.0 / K), mu, cov)
    for it in range(cfg["niter"]):
        new, so, (X, logw, flg, idx) = oracle.iterate_posterior(om, lpf, N, cfg["seed"], it, cfg["beta"], BMIN, BMAX,
                                                                want_sample=True)
        assert so["status"] == 0, so
        got = iters[it]
        assert got["nok"] == so["nok"], (it, got, so)
        for key in ("ln_evidence", "logSum"):
            assert abs(got[key] - so[key]) <= 1e-8 * max(1.0, abs(so[key])), (it, key, got[key], so[key])
        for key in ("perplexity", "ess", "enc"):
            assert abs(got[key] / so[key] - 1.0) <= 1e-6, (it, key, got[key], so[key])
        # the updated proposal (lower Cholesky factors)
        w = np.array([c[1] for c in comps[it]])
        np.testing.assert_allclose(w, new.w, rtol=1e-8, atol=1e-13)
        for k in np.flatnonzero(new.w > 0):
            chol, _, mk, Sk = comps[it][k]
            assert chol == 1
            ck = Sk @ Sk.T
            sd = np.sqrt(np.diag(new.cov[k]))
            assert np.max(np.abs(mk - new.mu[k]) / sd) < 1e-7, (it, k)
            assert np.max(np.abs(ck - new.cov[k]) / np.outer(sd, sd)) < 1e-7, (it, k)
        # the sample file: header with the par_t names, one row per counted sample
        path = tmp_path / f"pmcsim_{it}"
        head = [ln for ln in open(path) if ln.startswith("#")]
        assert head[0].startswith("# npar = 5, n_ded = 0")
        assert head[2].split()[1:] == ["Omega_m", "w_0_de", "M", "alpha", "beta"]
        rows = np.loadtxt(path, comments="#", ndmin=2)
        ok = flg == 1
        assert rows.shape == (int(ok.sum()), 2 + D)
        # the file holds log(normalised weight) + logSum, as the reference writes it
        # (exec/exec_helper.c:408-420): -inf where the normalised weight underflows,
        # fewer bits where it is subnormal (below 2.2e-308, log < -708.4)
        rel = logw[ok] - so["logSum"]
        fin = np.isfinite(rows[:, 0])
        assert np.all(rel[~fin] < -700.0)
        normal = rel > -708.0
        np.testing.assert_allclose(rows[normal, 0], logw[ok][normal], rtol=1e-8, atol=1e-8)
        np.testing.assert_allclose(rows[fin & ~normal, 0], logw[ok][fin & ~normal], rtol=0, atol=1.0)
        np.testing.assert_array_equal(rows[:, 1], -idx[ok].astype(float))
        np.testing.assert_allclose(rows[:, 2:], X[ok], rtol=1e-8, atol=1e-12)
        # continue from the C program's proposal
        L = np.array([comps[it][k][3] for k in range(K)])
        om = oracle.Mix(w, np.array([comps[it][k][2] for k in range(K)]), L=L)
